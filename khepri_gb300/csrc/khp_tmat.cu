// The tmat formulation of a patterned layer (khepri/tmat/scattering.py:25-51,
// matrices.py:126-212): the transfer matrix of a slice from the matrix exponential of the
// 4 ng x 4 ng field matrix A, turned into a scattering matrix and squared slicing_pow times by
// star products in the dense [p; m] layout (multS).
//
//   A (matrix_a, matrices.py:126-169): 4 x 4 blocks of ng x ng; diagonal blocks of the planar
//     wavevector u = kp + g and Toeplitz blocks eps_g[m_i - m_j + 2n], epsinv_g[...] of the
//     Fourier coefficients (harmonic g <-> (m1, m2) = (g % px - px/2, g / px - py/2));
//   E = expm(-A depth / 2^p): scaling and squaring with the degree-13 Pade approximant
//     (Higham, SIAM J. Matrix Anal. Appl. 26 (2005) 1179-1193), the batch's largest 1-norm
//     choosing one scaling for all problems; 6 products, one LU solve, s squarings;
//   T = U E Vi with U and Vi 4 x 4 blocks of diagonals (matrix_u / matrix_v,
//     matrices.py:9-74): 16 terms per element instead of two dense products;
//   S = matrix_s(T) (matrices.py:171-180), then S = multS(S, S) p times (matrices.py:194-212).
// Everything FP64 (the reference runs complex128 throughout).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "khepri_gb300.h"
#include "khp_core.cuh"
#include "khp_launch.h"

namespace khp {
namespace {

using cd = cplx<double>;

constexpr double kMu0c = 4.0 * 3.14159265358979323846 * 1e-7 * 299792458.0;  // constants.py:3-5
constexpr double kTwoPi = 6.28318530717958647692;

struct TArena2 {
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

// ---- field matrix A ------------------------------------------------------------------------
__global__ void k_tmat_a(int64_t batch, int px, int py, int nq0, int nq1, const cd* __restrict__ eps_g,
                         const cd* __restrict__ epsinv_g, const double* __restrict__ gx, const double* __restrict__ gy,
                         const double* __restrict__ kp, const double* __restrict__ wavelength, cd* A) {
  const int ng = px * py;
  const int64_t N = 4 * (int64_t)ng, NN = N * N;
  const int nx = px / 2, ny = py / 2;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < batch * NN; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / NN;
    const int64_t rc = e % NN;
    const int r = (int)(rc / N), c = (int)(rc % N);
    const int bi = r / ng, gi = r % ng, bj = c / ng, gj = c % ng;
    const double c1 = kTwoPi / wavelength[b];
    const cd ieo = mk(0.0, c1 / kMu0c), iseo = mk(0.0, kMu0c / c1), imo = mk(0.0, kMu0c * c1),
             ismo = mk(0.0, 1.0 / kMu0c / c1);
    const double uxi = kp[2 * b] + gx[gi], uyi = kp[2 * b + 1] + gy[gi];
    const double uxj = kp[2 * b] + gx[gj], uyj = kp[2 * b + 1] + gy[gj];
    const int i1 = (gi % px - nx) - (gj % px - nx) + 2 * nx;
    const int i2 = (gi / px - ny) - (gj / px - ny) + 2 * ny;
    const bool inq = i1 >= 0 && i1 < nq0 && i2 >= 0 && i2 < nq1;
    const cd ep = inq ? eps_g[(int64_t)i1 * nq1 + i2] : mk(0.0);
    const cd ei = inq ? epsinv_g[(int64_t)i1 * nq1 + i2] : mk(0.0);
    const bool diag = gi == gj;
    cd v = mk(0.0);
    const int blk = bi * 4 + bj;
    switch (blk) {
      case 8:  // (2, 0)
        if (diag) v = ismo * (-uxi * uyi);
        break;
      case 12:  // (3, 0)
        v = ieo * ep;
        if (diag) v += ismo * (-uyi * uyi);
        break;
      case 9:  // (2, 1)
        v = -(ieo * ep);
        if (diag) v += ismo * (uxi * uxi);
        break;
      case 13:  // (3, 1)
        if (diag) v = ismo * (uxi * uyi);
        break;
      case 6:  // (1, 2)
        v = iseo * ei * (uyi * uyj);
        if (diag) v -= imo;
        break;
      case 3:  // (0, 3)
        v = -(iseo * ei * (uxi * uxj));
        if (diag) v += imo;
        break;
      case 2:  // (0, 2)
        v = iseo * ei * (uxi * uyj);
        break;
      case 7:  // (1, 3)
        v = -(iseo * ei * (uyi * uxj));
        break;
      default:
        break;
    }
    A[e] = v;
  }
}

// ---- element-wise helpers --------------------------------------------------------------------
__global__ void k_scale(int64_t count, const cd* __restrict__ in, double s, cd* out) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < count; e += (int64_t)gridDim.x * blockDim.x)
    out[e] = in[e] * s;
}

// out = c1 X1 + c2 X2 + c3 X3 + c4 X4 + c0 I (any Xk may be null), per n x n matrix of a batch
__global__ void k_lincomb(int64_t batch, int n, double c0, double c1, const cd* X1, double c2, const cd* X2, double c3,
                          const cd* X3, double c4, const cd* X4, cd* out) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < batch * nn; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t rc = e % nn;
    cd v = mk((rc / n == rc % n) ? c0 : 0.0);
    if (X1) v += X1[e] * c1;
    if (X2) v += X2[e] * c2;
    if (X3) v += X3[e] * c3;
    if (X4) v += X4[e] * c4;
    out[e] = v;
  }
}

// Largest 1-norm (max column sum of |.|) over the batch, as an ordered-int atomic max.
__global__ void k_norm1_max(int64_t batch, int n, const cd* __restrict__ M, unsigned long long* out) {
  const int64_t cols = batch * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < cols; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / n;
    const int c = (int)(e % n);
    const cd* col = M + b * (int64_t)n * n + c;
    double s = 0.0;
    for (int r = 0; r < n; ++r) s += cabs(col[(int64_t)r * n]);
    if (!(s >= 0.0)) s = 1e308;  // NaN: flag through a huge norm (the solve then reports it)
    atomicMax(out, (unsigned long long)__double_as_longlong(s));
  }
}

// T = U E Vi with U, Vi given as 4 x 4 blocks of diagonals [batch][16][ng] (block (a, c) at a*4+c)
__global__ void k_tmat_uev(int64_t batch, int ng, const cd* __restrict__ u, const cd* __restrict__ E,
                           const cd* __restrict__ v, cd* T) {
  const int64_t N = 4 * (int64_t)ng, NN = N * N;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < batch * NN; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / NN;
    const int64_t rc = e % NN;
    const int r = (int)(rc / N), c = (int)(rc % N);
    const int a = r / ng, i = r % ng, bb = c / ng, j = c % ng;
    const cd* ub = u + b * 16 * ng;
    const cd* vb = v + b * 16 * ng;
    const cd* Eb = E + b * NN;
    cd acc = mk(0.0);
#pragma unroll
    for (int cc = 0; cc < 4; ++cc) {
      const cd uu = ub[(a * 4 + cc) * ng + i];
      cd inner = mk(0.0);
#pragma unroll
      for (int d = 0; d < 4; ++d) inner += Eb[(int64_t)(cc * ng + i) * N + d * ng + j] * vb[(d * 4 + bb) * ng + j];
      acc += uu * inner;
    }
    T[e] = acc;
  }
}

inline unsigned blocks_for(int64_t total) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, 152 * 32));
}

#define TM_TRY(x)       \
  do {                  \
    const int _s = (x); \
    if (_s) return _s;  \
  } while (0)
#define TM_EW(kernel, total, ...)                          \
  do {                                                     \
    kernel<<<blocks_for(total), 256, 0, s>>>(__VA_ARGS__); \
    count_launches(1);                                     \
    TM_TRY(cuda_status());                                 \
  } while (0)

// ---- matrix_s and multS in the dense [p; m] layout (h = 2 ng, N = 2 h) ----------------------
struct StarScratch {
  cd *lu, *R, *X1, *X2;
  int* piv;
};

template <class Arena>
StarScratch plan_star(Arena& a, int64_t batch, int h) {
  const size_t hh = (size_t)h * h;
  StarScratch p;
  p.lu = a.template take<cd>(batch * hh);
  p.R = a.template take<cd>(batch * 2 * hh);
  p.X1 = a.template take<cd>(batch * hh);
  p.X2 = a.template take<cd>(batch * hh);
  p.piv = a.template take<int>(batch * h);
  return p;
}

int matrix_s(int64_t batch, int h, const cd* T, cd* S, const StarScratch& w, int* status, cudaStream_t s) {
  const int N = 2 * h;
  const int64_t NN = (int64_t)N * N, hh = (int64_t)h * h;
  const cd one = mk(1.0), mone = mk(-1.0), zero = mk(0.0);
  const cd* Tpp = T;
  const cd* Tpm = T + h;
  const cd* Tmp = T + (int64_t)h * N;
  const cd* Tmm = T + (int64_t)h * N + h;
  cd* Spp = S;
  cd* Spm = S + h;
  cd* Smp = S + (int64_t)h * N;
  cd* Smm = S + (int64_t)h * N + h;
  TM_TRY(launch_copy<double>(batch, h, h, Tpp, N, NN, w.lu, h, hh, s));
  TM_TRY(launch_inverse_blocked<double>(batch, h, w.lu, h, hh, Spp, N, NN, w.piv, status, s));
  TM_TRY(launch_gemm<double>(batch, h, h, h, mone, Spp, N, NN, Tpm, N, NN, zero, Spm, N, NN, s));
  TM_TRY(launch_gemm<double>(batch, h, h, h, one, Tmp, N, NN, Spp, N, NN, zero, Smp, N, NN, s));
  TM_TRY(launch_copy<double>(batch, h, h, Tmm, N, NN, Smm, N, NN, s));
  TM_TRY(launch_gemm<double>(batch, h, h, h, one, Tmp, N, NN, Spm, N, NN, one, Smm, N, NN, s));
  return KHP_OK;
}

int mult_s(int64_t batch, int h, const cd* S1, int64_t bs1, const cd* S2, int64_t bs2, cd* S, const StarScratch& w,
           int* status, cudaStream_t s) {
  const int N = 2 * h;
  const int64_t NN = (int64_t)N * N, hh = (int64_t)h * h;
  const cd one = mk(1.0), mone = mk(-1.0), zero = mk(0.0);
  auto blk = [&](const cd* M, int r, int c) { return M + (int64_t)r * h * N + c * h; };
  cd* Spp = S;
  cd* Spm = S + h;
  cd* Smp = S + (int64_t)h * N;
  cd* Smm = S + (int64_t)h * N + h;
  // I = I0 - S1pm S2mp ; R = [S1pp | S1pm] ; R <- I^-1 R = [G1 | G2]
  TM_TRY(launch_identity<double>(batch, h, h, w.lu, h, hh, one, s));
  TM_TRY(launch_gemm<double>(batch, h, h, h, mone, blk(S1, 0, 1), N, bs1, blk(S2, 1, 0), N, bs2, one, w.lu, h, hh, s));
  TM_TRY(launch_copy<double>(batch, h, h, blk(S1, 0, 0), N, bs1, w.R, 2 * h, 2 * hh, s));
  TM_TRY(launch_copy<double>(batch, h, h, blk(S1, 0, 1), N, bs1, w.R + h, 2 * h, 2 * hh, s));
  TM_TRY(launch_getrf_blocked<double>(batch, h, w.lu, h, hh, w.piv, status, s));
  TM_TRY(launch_getrs_blocked<double>(batch, h, w.lu, h, hh, w.piv, w.R, 2 * h, 2 * hh, 2 * h, s));
  const cd* G1 = w.R;
  const cd* G2 = w.R + h;
  // S[p,p] = S2pp G1
  TM_TRY(launch_gemm<double>(batch, h, h, h, one, blk(S2, 0, 0), N, bs2, G1, 2 * h, 2 * hh, zero, Spp, N, NN, s));
  // S[m,p] = S1mp + S1mm (S2mp G1)
  TM_TRY(launch_gemm<double>(batch, h, h, h, one, blk(S2, 1, 0), N, bs2, G1, 2 * h, 2 * hh, zero, w.X1, h, hh, s));
  TM_TRY(launch_copy<double>(batch, h, h, blk(S1, 1, 0), N, bs1, Smp, N, NN, s));
  TM_TRY(launch_gemm<double>(batch, h, h, h, one, blk(S1, 1, 1), N, bs1, w.X1, h, hh, one, Smp, N, NN, s));
  // X2 = G2 S2mm ; S[p,m] = S2pm + S2pp X2
  TM_TRY(launch_gemm<double>(batch, h, h, h, one, G2, 2 * h, 2 * hh, blk(S2, 1, 1), N, bs2, zero, w.X2, h, hh, s));
  TM_TRY(launch_copy<double>(batch, h, h, blk(S2, 0, 1), N, bs2, Spm, N, NN, s));
  TM_TRY(launch_gemm<double>(batch, h, h, h, one, blk(S2, 0, 0), N, bs2, w.X2, h, hh, one, Spm, N, NN, s));
  // S[m,m] = S1mm (S2mm + S2mp X2)
  TM_TRY(launch_copy<double>(batch, h, h, blk(S2, 1, 1), N, bs2, w.X1, h, hh, s));
  TM_TRY(launch_gemm<double>(batch, h, h, h, one, blk(S2, 1, 0), N, bs2, w.X2, h, hh, one, w.X1, h, hh, s));
  TM_TRY(launch_gemm<double>(batch, h, h, h, one, blk(S1, 1, 1), N, bs1, w.X1, h, hh, zero, Smm, N, NN, s));
  return KHP_OK;
}

// ---- layer plan -----------------------------------------------------------------------------
struct LayerPlan {
  cd *A, *M, *M2, *M4, *M6, *W, *Z, *P, *Q, *E, *T, *S2;
  int* piv;
  unsigned long long* norm;
  StarScratch star;
};

template <class Arena>
LayerPlan plan_layer(Arena& a, int64_t batch, int ng) {
  const size_t N = 4 * (size_t)ng, NN = N * N;
  LayerPlan p;
  p.A = a.template take<cd>(batch * NN);
  p.M = a.template take<cd>(batch * NN);
  p.M2 = a.template take<cd>(batch * NN);
  p.M4 = a.template take<cd>(batch * NN);
  p.M6 = a.template take<cd>(batch * NN);
  p.W = a.template take<cd>(batch * NN);
  p.Z = a.template take<cd>(batch * NN);
  p.P = a.template take<cd>(batch * NN);
  p.Q = a.template take<cd>(batch * NN);
  p.E = a.template take<cd>(batch * NN);
  p.T = a.template take<cd>(batch * NN);
  p.S2 = a.template take<cd>(batch * NN);
  p.piv = a.template take<int>(batch * N);
  p.norm = a.template take<unsigned long long>(1);
  p.star = plan_star(a, batch, 2 * ng);
  return p;
}

// Pade-13 coefficients b_0 .. b_13 of the exponential (Higham 2005, eq. 2.3 with m = 13).
constexpr double kPade13[14] = {64764752532480000.0, 32382376266240000.0, 7771770303897600.0, 1187353796428800.0,
                                129060195264000.0,   10559470521600.0,    670442572800.0,     33522128640.0,
                                1323241920.0,        40840800.0,          960960.0,           16380.0,
                                182.0,               1.0};
constexpr double kTheta13 = 5.371920351148152;

// E = expm(M) for every matrix of the batch (M is overwritten).
int expm_batched(int64_t batch, int N, LayerPlan& p, int* status, cudaStream_t s) {
  const int64_t NN = (int64_t)N * N;
  const cd one = mk(1.0), zero = mk(0.0);
  if (cudaMemsetAsync(p.norm, 0, sizeof(unsigned long long), s) != cudaSuccess) return KHP_ERR_CUDA;
  TM_EW(k_norm1_max, batch * N, batch, N, p.M, p.norm);
  unsigned long long bits = 0;
  if (cudaMemcpyAsync(&bits, p.norm, sizeof(bits), cudaMemcpyDeviceToHost, s) != cudaSuccess) return KHP_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return KHP_ERR_CUDA;
  double nrm;
  static_assert(sizeof(nrm) == sizeof(bits), "bit copy");
  std::memcpy(&nrm, &bits, sizeof(nrm));
  if (!(nrm < 1e300)) return KHP_ERR_NONFINITE;
  int sq = 0;
  if (nrm > kTheta13) sq = (int)std::ceil(std::log2(nrm / kTheta13));
  if (sq > 1000) return KHP_ERR_NONFINITE;
  if (sq > 0) TM_EW(k_scale, batch * NN, batch * NN, p.M, std::ldexp(1.0, -sq), p.M);
  const double* b = kPade13;
  TM_TRY(launch_gemm<double>(batch, N, N, N, one, p.M, N, NN, p.M, N, NN, zero, p.M2, N, NN, s));
  TM_TRY(launch_gemm<double>(batch, N, N, N, one, p.M2, N, NN, p.M2, N, NN, zero, p.M4, N, NN, s));
  TM_TRY(launch_gemm<double>(batch, N, N, N, one, p.M4, N, NN, p.M2, N, NN, zero, p.M6, N, NN, s));
  // U = M [M6 (b13 M6 + b11 M4 + b9 M2) + b7 M6 + b5 M4 + b3 M2 + b1 I]
  TM_EW(k_lincomb, batch * NN, batch, N, 0.0, b[13], p.M6, b[11], p.M4, b[9], p.M2, 0.0, nullptr, p.W);
  TM_TRY(launch_gemm<double>(batch, N, N, N, one, p.M6, N, NN, p.W, N, NN, zero, p.Z, N, NN, s));
  TM_EW(k_lincomb, batch * NN, batch, N, b[1], 1.0, p.Z, b[7], p.M6, b[5], p.M4, b[3], p.M2, p.W);
  TM_TRY(launch_gemm<double>(batch, N, N, N, one, p.M, N, NN, p.W, N, NN, zero, p.P, N, NN, s));  // P = U
  // V = M6 (b12 M6 + b10 M4 + b8 M2) + b6 M6 + b4 M4 + b2 M2 + b0 I
  TM_EW(k_lincomb, batch * NN, batch, N, 0.0, b[12], p.M6, b[10], p.M4, b[8], p.M2, 0.0, nullptr, p.W);
  TM_TRY(launch_gemm<double>(batch, N, N, N, one, p.M6, N, NN, p.W, N, NN, zero, p.Z, N, NN, s));
  TM_EW(k_lincomb, batch * NN, batch, N, b[0], 1.0, p.Z, b[6], p.M6, b[4], p.M4, b[2], p.M2, p.W);  // W = V
  // (V - U) E = V + U
  TM_EW(k_lincomb, batch * NN, batch, N, 0.0, 1.0, p.W, -1.0, p.P, 0.0, nullptr, 0.0, nullptr, p.Q);
  TM_EW(k_lincomb, batch * NN, batch, N, 0.0, 1.0, p.W, 1.0, p.P, 0.0, nullptr, 0.0, nullptr, p.E);
  TM_TRY(launch_getrf_blocked<double>(batch, N, p.Q, N, NN, p.piv, status, s));
  TM_TRY(launch_getrs_blocked<double>(batch, N, p.Q, N, NN, p.piv, p.E, N, NN, N, s));
  for (int k = 0; k < sq; ++k) {
    TM_TRY(launch_gemm<double>(batch, N, N, N, one, p.E, N, NN, p.E, N, NN, zero, p.Z, N, NN, s));
    std::swap(p.E, p.Z);
  }
  return KHP_OK;
}

}  // namespace
}  // namespace khp

using namespace khp;

extern "C" {

size_t khp_tmat_layer_workspace(int64_t batch, int32_t ng) {
  if (batch < 0 || ng < 1) return 0;
  TArena2 a{nullptr, 0};
  plan_layer(a, batch, ng);
  return a.off;
}

int khp_tmat_layer_smatrix(int64_t batch, int32_t px, int32_t py, int32_t nq0, int32_t nq1, const double* eps_g,
                           const double* epsinv_g, const double* gx, const double* gy, const double* kp,
                           const double* wavelength, const double* u_blocks, const double* v_blocks, double depth,
                           int32_t slicing_pow, double* S, double* A_out, double* E_out, double* T_out,
                           int32_t* status, void* workspace, size_t ws_bytes, void* stream) {
  if (batch < 0 || px < 1 || py < 1 || nq0 < 1 || nq1 < 1 || slicing_pow < 0 || slicing_pow > 60 || !eps_g ||
      !epsinv_g || !gx || !gy || !kp || !wavelength || !u_blocks || !v_blocks || !S || !status)
    return KHP_ERR_INVALID_ARG;
  if (batch == 0) return KHP_OK;
  const int ng = px * py;
  TArena2 a{static_cast<char*>(workspace), ws_bytes};
  LayerPlan p = plan_layer(a, batch, ng);
  if (!a.ok || !workspace) return KHP_ERR_WORKSPACE;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const int N = 4 * ng, h = 2 * ng;
  const int64_t NN = (int64_t)N * N;
  cd* A = A_out ? reinterpret_cast<cd*>(A_out) : p.A;
  TM_EW(k_tmat_a, batch * NN, batch, px, py, nq0, nq1, reinterpret_cast<const cd*>(eps_g),
        reinterpret_cast<const cd*>(epsinv_g), gx, gy, kp, wavelength, A);
  TM_EW(k_scale, batch * NN, batch * NN, A, -depth / std::ldexp(1.0, slicing_pow), p.M);
  TM_TRY(expm_batched(batch, N, p, status, s));
  if (E_out) TM_TRY(launch_copy<double>(batch, N, N, p.E, N, NN, reinterpret_cast<cd*>(E_out), N, NN, s));
  cd* T = T_out ? reinterpret_cast<cd*>(T_out) : p.T;
  TM_EW(k_tmat_uev, batch * NN, batch, ng, reinterpret_cast<const cd*>(u_blocks), p.E,
        reinterpret_cast<const cd*>(v_blocks), T);
  // S = matrix_s(T), then S = multS(S, S) slicing_pow times (ping-pong with the scratch S2)
  cd* cur = (slicing_pow % 2 == 0) ? reinterpret_cast<cd*>(S) : p.S2;
  cd* oth = (slicing_pow % 2 == 0) ? p.S2 : reinterpret_cast<cd*>(S);
  TM_TRY(matrix_s(batch, h, T, cur, p.star, status, s));
  for (int k = 0; k < slicing_pow; ++k) {
    TM_TRY(mult_s(batch, h, cur, NN, cur, NN, oth, p.star, status, s));
    std::swap(cur, oth);
  }
  return cuda_status();
}

int khp_tmat_matrix_s(int64_t batch, int32_t ng, const double* T, double* S, int32_t* status, void* workspace,
                      size_t ws_bytes, void* stream) {
  if (batch < 0 || ng < 1 || !T || !S || !status) return KHP_ERR_INVALID_ARG;
  if (batch == 0) return KHP_OK;
  TArena2 a{static_cast<char*>(workspace), ws_bytes};
  StarScratch w = plan_star(a, batch, 2 * ng);
  if (!a.ok || !workspace) return KHP_ERR_WORKSPACE;
  const int st = matrix_s(batch, 2 * ng, reinterpret_cast<const cd*>(T), reinterpret_cast<cd*>(S), w, status,
                          reinterpret_cast<cudaStream_t>(stream));
  return st ? st : cuda_status();
}

size_t khp_tmat_multS_workspace(int64_t batch, int32_t ng) {
  if (batch < 0 || ng < 1) return 0;
  TArena2 a{nullptr, 0};
  plan_star(a, batch, 2 * ng);
  return a.off;
}

int khp_tmat_multS(int64_t batch, int32_t ng, const double* S1, int64_t s1_stride, const double* S2, int64_t s2_stride,
                   double* S, int32_t* status, void* workspace, size_t ws_bytes, void* stream) {
  if (batch < 0 || ng < 1 || !S1 || !S2 || !S || !status) return KHP_ERR_INVALID_ARG;
  const int64_t NN = 16 * (int64_t)ng * ng;
  if (s1_stride < NN || s2_stride < NN) return KHP_ERR_INVALID_ARG;
  if (batch == 0) return KHP_OK;
  TArena2 a{static_cast<char*>(workspace), ws_bytes};
  StarScratch w = plan_star(a, batch, 2 * ng);
  if (!a.ok || !workspace) return KHP_ERR_WORKSPACE;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const int st = mult_s(batch, 2 * ng, reinterpret_cast<const cd*>(S1), s1_stride, reinterpret_cast<const cd*>(S2),
                        s2_stride, reinterpret_cast<cd*>(S), w, status, s);
  return st ? st : cuda_status();
}

}  // extern "C"
