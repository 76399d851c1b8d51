// Mixed-precision batched R/T (khp_solve_batched_mixed): FP32 for every O(n^3) step, FP64 only
// where accuracy is decided.
//
// GB300 runs FP32 at ~58x its FP64 rate, but an all-FP32 solve misses |dR|, |dT| <= 1e-6 (errors
// of a few 1e-6 on the 11x11 sweep).  This pipeline:
//   1. modes: FP32 eigensolve of M = P Q, then three FP64 refinement steps of the eigenpairs:
//      E = W^-1 (M W - W mu) with the residual formed in FP64 and the solve in FP32,
//      mu += diag(E), W += W F with F_ij = E_ij / (mu_j - mu_i); clusters of eigenvalues closer
//      than 1e-3 max|mu| take the exact eigen-decomposition of their block of diag(mu) + E
//      instead (cyclic 2x2 Jacobi sweeps), composed with the first-order correction of their
//      columns; an FP64 residual test of every mode follows (status bit 32 where it fails);
//      V = Q W / lam in FP64.  The FP64 products M W and C W run on the bf16 tensor cores with
//      exact digit splitting (ozaki_zgemm), FP64-accurate;
//   2. the reflection-matrix recursion of khp_solve_batched on the FP32-rounded refined modes,
//      keeping every factor it makes (the explicit inverses, rho, Gamma at every gap, Gamma M^-1),
//      with every O(n^3) step a blocked LU / inverse or a tiled product;
//   3. iterative refinement of the interface-continuity system of the whole stack (the
//      equations the reference's S-matrix chain encodes, crystal.py:180-206 / layer.py:35-60),
//      for the two source columns: residual in FP64 with the refined FP64 modes and the FP64
//      closed-form homogeneous blocks (O(n^2) per layer), correction by an affine sweep through
//      the kept FP32 factors (O(n^2) per layer).
// The converged amplitudes solve the FP64 system; R and T follow as in crystal.py:363-396.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "khepri_gb300.h"
#include "khp_dense.cuh"
#include "khp_gamma_kernels.cuh"
#include "khp_launch.h"
#include "khp_physics.cuh"

namespace khp {
namespace {

using cf = cplx<float>;

constexpr int kMaxLayers = 16;
// Eigen-refinement steps.  From this FP32 solver's eigenvectors (relative residual ~1e-6 on the
// 11x11 P.Q) three cluster-aware steps with M W formed in FP64 at every step reach ~1e-15, also
// for exactly degenerate pairs and for clusters of close eigenvalues.
constexpr int kEigSteps = 3;
// Refinement rounds beyond the requested ones, run only for problems not yet converged.
constexpr int kExtraRounds = 12;
// Largest refine_iters the entry points accept (every round is one residual and one sweep launch).
constexpr int kMaxRefine = 64;

// ------------------------------------------------------------------------------------------
// Eigen-refinement kernels
// ------------------------------------------------------------------------------------------
// R32 = (M64 W64 - W64 diag(mu)) in FP32, where MW already holds M64 W64.
// One grid row per problem (b = boff + blockIdx.y), launched by MX_PP.
__global__ void k_eig_residual(int64_t boff, int n, const cd* __restrict__ MW, const cd* __restrict__ W64,
                               const cd* __restrict__ mu, cf* R32) {
  const int64_t nn = (int64_t)n * n;
  const int64_t b = boff + blockIdx.y;
  for (int rc = blockIdx.x * blockDim.x + threadIdx.x; rc < nn; rc += gridDim.x * blockDim.x) {
    const int64_t e = b * nn + rc;
    const int j = rc % n;
    const cd r = MW[e] - W64[e] * mu[b * n + j];
    R32[e] = mk((float)r.re, (float)r.im);
  }
}

// The 2x2 eigen-decomposition of K = [[a, b], [c, d]] with eigenvectors scaled to unit
// diagonal: returns den with v12 = -b/den, v21 = c/den, new eigenvalues a + bc/den and
// d - bc/den (the root near a first).
__device__ __forceinline__ cd pair_den(cd a, cd b, cd c, cd d) {
  const cd h = 0.5 * (a - d);
  const cd sq = csqrt(h * h + b * c);
  return (h.re * sq.re + h.im * sq.im >= 0.0) ? h + sq : h - sq;
}

// Eigenvalue clusters of the refinement: the connected components of the graph joining
// eigenvalues closer than kClusterTol max|mu|.  Inside a cluster a first-order step converges
// slowly or not at all (its correction E_ij / (mu_j - mu_i) is not small), so every cluster of
// 2..kClusterMax members takes the exact eigen-decomposition of its block of diag(mu) + E instead.
// A component larger than kClusterMax (a chain of close eigenvalues) is split again at a third of
// the distance, up to kClusterLevels times; what is still too large is treated member by member.
constexpr double kClusterTol = 1e-3;
constexpr int kClusterMax = 12;
constexpr int kClusterLevels = 4;
// Cluster members whose 2x2 sub-block does not resolve two directions (|den| below this times
// max|mu|) are degenerate to within the refinement's noise (e.g. the two modes of a
// two-dimensional representation of a symmetric pixmap at normal incidence): any basis of an
// exactly degenerate subspace is an eigenbasis, and a rotation computed from noise is O(1).
constexpr double kDegenerateTol = 1e-9;

// Cyclic 2x2 Jacobi sweeps for a non-normal k x k matrix K close to diagonal: each step is the
// similarity S^-1 K S with S = [[1, v12], [v21, 1]] on rows and columns (a, b), the 2x2 block's
// eigenvectors scaled to unit diagonal, which zeroes K_ab and K_ba; X accumulates the S.  Pairs
// degenerate within the noise, or whose S is nearly singular, are left alone.  At most 16 sweeps,
// stopping once every off-diagonal entry is below 1e-15 max|mu|.
__device__ void cluster_jacobi(int k, cd* K, cd* X, double big) {
  for (int i = 0; i < k * k; ++i) X[i] = mk(0.0);
  for (int i = 0; i < k; ++i) X[i * k + i] = mk(1.0);
  for (int sweep = 0; sweep < 16; ++sweep) {
    double off = 0.0;
    for (int a = 0; a < k; ++a) {
      for (int b = a + 1; b < k; ++b) {
        const cd kab = K[a * k + b], kba = K[b * k + a];
        off = fmax(off, fmax(cabs(kab), cabs(kba)));
        const cd den = pair_den(K[a * k + a], kab, kba, K[b * k + b]);
        if (!(cabs(den) > kDegenerateTol * big)) continue;
        const cd v12 = cdiv(mk(-kab.re, -kab.im), den), v21 = cdiv(kba, den);
        const cd det = mk(1.0) - v12 * v21;
        if (!(cabs(det) > 1e-3)) continue;
        const cd idet = cdiv(mk(1.0), det);
        // columns a, b of K and X: [ca, cb] <- [ca + v21 cb, cb + v12 ca]
        for (int r = 0; r < k; ++r) {
          const cd ca = K[r * k + a], cb = K[r * k + b];
          K[r * k + a] = ca + v21 * cb;
          K[r * k + b] = cb + v12 * ca;
          const cd xa = X[r * k + a], xb = X[r * k + b];
          X[r * k + a] = xa + v21 * xb;
          X[r * k + b] = xb + v12 * xa;
        }
        // rows a, b of K: [ra; rb] <- (1 / det) [ra - v12 rb; rb - v21 ra]
        for (int c = 0; c < k; ++c) {
          const cd ra = K[a * k + c], rb = K[b * k + c];
          K[a * k + c] = idet * (ra - v12 * rb);
          K[b * k + c] = idet * (rb - v21 * ra);
        }
      }
    }
    if (off < 1e-15 * big) break;
  }
}

// Clusters of one refinement step (one CTA per problem).  Writes, per column j: lab[j] (the
// smallest index of its cluster), pos[j] (its rank among the members), csz[j] (the cluster size,
// 1 for a singleton), the updated eigenvalue mu_out[j], and for members of clusters of size
// 2..kClusterMax the members (memb[j][p]) and column pos[j] of the cluster's transform
// (xc[j][p] = X[p][pos[j]]).  Columns of larger clusters are treated as singletons.
__global__ void __launch_bounds__(256) k_clusters(int n, const cd* __restrict__ mu, const cf* __restrict__ E,
                                                  int* lab, int* pos, int* csz, int* memb, cf* xc, cd* mu_out) {
  __shared__ TeamShared sh;
  __shared__ int changed;
  TeamCta t;
  const int64_t b = blockIdx.x;
  const int64_t nn = (int64_t)n * n;
  const cd* m = mu + b * n;
  const cf* Eb = E + b * nn;
  int* lb = lab + b * n;
  double big = 0.0;
  int bi = 0;
  for (int i = t.tid(); i < n; i += t.size()) {
    big = fmax(big, cabs(m[i]));
    lb[i] = i;
  }
  team_argmax(t, big, bi, &sh);
  int* sz = csz + b * n;
  int* act = pos + b * n;  // scratch until the ranks are written: column still being split
  double tol = kClusterTol * big;
  for (int level = 0; level < kClusterLevels; ++level, tol *= (1.0 / 3.0)) {
    if (t.tid() == 0) changed = 0;
    t.sync();
    for (int i = t.tid(); i < n; i += t.size()) {
      act[i] = level == 0 || sz[i] > kClusterMax;
      if (act[i]) {
        lb[i] = i;
        changed = 1;
      }
    }
    t.sync();
    if (!changed) break;
    t.sync();
    const double tol2 = tol * tol;
    // connected components among the columns being split, by repeated minimum-label propagation
    // (bounded; a component whose labels have not settled is only split further, and each part is
    // still handled consistently)
    for (int it = 0; it < 64; ++it) {
      if (t.tid() == 0) changed = 0;
      t.sync();
      for (int i = t.tid(); i < n; i += t.size()) {
        if (!act[i]) continue;
        const cd mi = m[i];
        int best = lb[i];
        for (int j = 0; j < n; ++j) {
          if (!act[j]) continue;
          const double dr = m[j].re - mi.re, di = m[j].im - mi.im;
          if (dr * dr + di * di < tol2) best = min(best, lb[j]);
        }
        if (best < lb[i]) {
          lb[i] = best;
          changed = 1;
        }
      }
      t.sync();
      if (!changed) break;
      t.sync();
    }
    // component sizes of the columns just labelled (a label is the smallest index of its
    // component, so it never equals the label of a column outside it)
    for (int i = t.tid(); i < n; i += t.size()) {
      if (!act[i]) continue;
      int c = 0;
      for (int j = 0; j < n; ++j) c += lb[j] == lb[i];
      sz[i] = c;
    }
    t.sync();
  }
  // ranks (deterministic: by index)
  for (int i = t.tid(); i < n; i += t.size()) {
    const int l = lb[i];
    int r = 0;
    for (int j = 0; j < i; ++j) r += lb[j] == l;
    pos[b * n + i] = r;
    const cf e = Eb[(int64_t)i * n + i];
    mu_out[b * n + i] = m[i] + mk((double)e.re, (double)e.im);
  }
  t.sync();
  // one thread per cluster of 2..kClusterMax members
  for (int r = t.tid(); r < n; r += t.size()) {
    if (lb[r] != r) continue;
    const int k = csz[b * n + r];
    if (k < 2 || k > kClusterMax) continue;
    int mem[kClusterMax];
    cd K[kClusterMax * kClusterMax], X[kClusterMax * kClusterMax];
    int c = 0;
    for (int j = r; j < n && c < k; ++j)
      if (lb[j] == r) mem[c++] = j;
    for (int p = 0; p < k; ++p)
      for (int q = 0; q < k; ++q) {
        const cf e = Eb[(int64_t)mem[p] * n + mem[q]];
        K[p * k + q] = mk((double)e.re, (double)e.im) + (p == q ? m[mem[p]] : mk(0.0));
      }
    cluster_jacobi(k, K, X, big);
    for (int q = 0; q < k; ++q) {
      const int j = mem[q];
      mu_out[b * n + j] = K[q * k + q];
      for (int p = 0; p < k; ++p) {
        memb[(b * n + j) * kClusterMax + p] = mem[p];
        xc[(b * n + j) * kClusterMax + p] = mk((float)X[p * k + q].re, (float)X[p * k + q].im);
      }
    }
  }
}

// First-order coefficient E_ik / (mu_k - mu_i) of column k's correction along column i (0 for
// eigenvalues closer than 1e-5 relative, which stay coupled: their error is second order).  The
// difference is taken in FP64 (no cancellation for close pairs), the quotient in FP32.
__device__ __forceinline__ cf first_order(const cf* Eb, const cd* mb, int n, int i, int k) {
  const cd mi = mb[i], mkk = mb[k];
  const cd dd = mkk - mi;
  const cf d32 = mk((float)dd.re, (float)dd.im);
  const float ad = cabs(d32);
  const float am = cabs(mk((float)mi.re, (float)mi.im)) + cabs(mk((float)mkk.re, (float)mkk.im));
  return ad > 1e-5f * am ? cdiv(Eb[(int64_t)i * n + k], d32) : mk(0.f);
}

// F of one refinement step, W += W F (one grid row per problem, b = boff + blockIdx.y, launched
// by MX_PP).  A singleton column j: F_ij = E_ij / (mu_j - mu_i).  A column j of a cluster C with
// transform X: the composition (I + F1) X - I of the first-order correction F1 of the cluster's
// columns and X, that is F_ij = sum_{c in C} F1_ic X_cj for i outside C and X_ij - delta_ij
// inside.  Applying X to uncorrected columns instead would leave a share of the other members'
// first-order errors in column j, and the step would not converge for clustered eigenvalues.
__global__ void k_eig_update(int64_t boff, int n, const cd* __restrict__ mu_in, const cf* __restrict__ E, cf* F,
                             const int* __restrict__ lab, const int* __restrict__ pos, const int* __restrict__ csz,
                             const int* __restrict__ memb, const cf* __restrict__ xc) {
  const int64_t nn = (int64_t)n * n;
  const int64_t b = boff + blockIdx.y;
  const cf* Eb = E + b * nn;
  const cd* mb = mu_in + b * n;
  for (int rc = blockIdx.x * blockDim.x + threadIdx.x; rc < nn; rc += gridDim.x * blockDim.x) {
    const int i = rc / n, j = rc - i * n;
    const int k = csz[b * n + j];
    cf out = mk(0.f);
    if (k < 2 || k > kClusterMax) {
      if (i != j) out = first_order(Eb, mb, n, i, j);
    } else {
      const int64_t cj = (b * n + j) * kClusterMax;
      if (lab[b * n + i] == lab[b * n + j]) {
        out = xc[cj + pos[b * n + i]];
        if (i == j) out.re -= 1.f;
      } else {
        for (int p = 0; p < k; ++p) fma_acc(out, first_order(Eb, mb, n, i, memb[cj + p]), xc[cj + p]);
      }
    }
    F[b * nn + rc] = out;
  }
}

// R and T of a problem are undefined when its incident wave is evanescent: the incident kz is
// imaginary (Re kz_inc = 0), the flux normalisation divides by it and both come out NaN, as in
// the reference (crystal.py:363-396, alternative.py:235-245).  Such a problem is never flagged for
// a re-solve, which could not change them.
__device__ __forceinline__ bool rt_undefined(const double* kp, double k0, cd epsi) {
  const cd kpx = mk(kp[0], kp[1]), kpy = mk(kp[2], kp[3]);
  return conj(csqrt(mk(k0 * k0) * epsi - kpx * kpx - kpy * kpy)).re == 0.0;
}

// Eigen-residual check after the last refinement step: MW holds M W (FP64-accurate).  A problem
// whose relative residual max_i |(M W - W diag(mu))_ij| / (max|mu| max_i |W_ij|) exceeds 1e-8 in
// any column j, or is not finite, gets KHP_BIT_MODES (unless its R and T are undefined).  One CTA
// per matrix; lanes take consecutive columns, so each row's loads are coalesced.
__global__ void __launch_bounds__(256) k_eig_check(int n, const cd* __restrict__ MW, const cd* __restrict__ W,
                                                   const cd* __restrict__ mu, const double* __restrict__ kp,
                                                   const double* __restrict__ k0, cd epsi, int* stat) {
  __shared__ TeamShared sh;
  TeamCta t;
  const int64_t b = blockIdx.x;
  if (rt_undefined(kp + 4 * b, k0[b], epsi)) return;
  const int64_t nn = (int64_t)n * n;
  const cd* mb = mu + b * n;
  double big = 0.0;
  int bi = 0;
  for (int i = t.tid(); i < n; i += t.size()) big = fmax(big, cabs(mb[i]));
  team_argmax(t, big, bi, &sh);
  double worst = 0.0;
  for (int j = t.tid(); j < n; j += t.size()) {
    double r = 0.0, w = 0.0;
    const cd mj = mb[j];
    for (int i = 0; i < n; ++i) {
      const int64_t e = b * nn + (int64_t)i * n + j;
      const cd wij = W[e];
      r = fmax(r, cabs(MW[e] - wij * mj));
      w = fmax(w, cabs(wij));
    }
    const double rel = r / (big * w);
    worst = rel == rel ? fmax(worst, rel) : INFINITY;  // a NaN fails the test
  }
  team_argmax(t, worst, bi, &sh);
  if (t.tid() == 0 && !(worst <= 1e-8)) stat[b] |= KHP_BIT_MODES;
}

// W64 += D32 ; W32 = round(W64)
__global__ void k_add_correction(int64_t count, cd* W64, const cf* __restrict__ D, cf* W32) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < count; e += (int64_t)gridDim.x * blockDim.x) {
    const cd w = W64[e] + mk((double)D[e].re, (double)D[e].im);
    W64[e] = w;
    W32[e] = mk((float)w.re, (float)w.im);
  }
}

__global__ void k_to_double(int64_t count, const cf* __restrict__ in, cd* out) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < count; e += (int64_t)gridDim.x * blockDim.x)
    out[e] = mk((double)in[e].re, (double)in[e].im);
}

// lam64 = sqrt(mu64), lam32 = round(lam64).  Principal root (alternative.py:173), except that a
// root within 1e-8 relative of the imaginary axis is taken with Im >= 0: mu on (or rounded
// across) the negative real axis then gets one branch, so that degenerate propagating pairs
// share it.  The sign of a mode's lam does not change the layer's scattering (the pair +-lam
// spans the same fields), and the gradient's divided differences need the shared branch.
__global__ void k_sqrt_mu(int64_t count, const cd* __restrict__ mu64, cd* lam64, cf* lam32) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < count; e += (int64_t)gridDim.x * blockDim.x) {
    cd l = csqrt(mu64[e]);
    if (fabs(l.re) <= 1e-8 * cabs(l) && l.im < 0.0) l = mk(-l.re, -l.im);
    lam64[e] = l;
    lam32[e] = mk((float)l.re, (float)l.im);
  }
}

// Per-matrix copies of kp ([batch][2] complex) and k0 for the slot-major modes batch.
__global__ void k_expand_problems(int64_t total, int64_t batch, int S, const double* __restrict__ kp,
                                  const double* __restrict__ k0, double* kpx, double* k0x) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < total; v += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = v % batch;
    for (int q = 0; q < 4; ++q) kpx[4 * v + q] = kp[4 * b + q];
    k0x[v] = k0[b];
  }
}

// status[b] |= statx[m][b] over the S slots.
__global__ void k_or_status(int64_t batch, int S, const int* __restrict__ statx, int* status) {
  for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < batch; b += (int64_t)gridDim.x * blockDim.x) {
    int w = 0;
    for (int m = 0; m < S; ++m) w |= statx[(int64_t)m * batch + b];
    status[b] |= w;
  }
}

// The loss seeds of problems whose stack refinement did not converge (status bit 8) cleared, so
// that they add nothing to the map gradients (GR, GT: [batch][2n]); the caller solves them again
// with more rounds and adds their share.
__global__ void k_drop_unconverged_seeds(int64_t batch, int n2, const int* __restrict__ status, cd* GR, cd* GT) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < batch * n2; e += (int64_t)gridDim.x * blockDim.x) {
    if (status[e / n2] & KHP_BIT_REFINE) {
      GR[e] = mk(0.0);
      GT[e] = mk(0.0);
    }
  }
}

// ---- double-float arithmetic for the stack residual's FP64 products ----------------------
// A double d is carried as hi + lo, hi = fl32(d), lo = fl32(d - hi): about 48 significant bits
// (the accumulation keeps ~1e-12 of the sum).  That is enough for the refinement rounds every
// problem runs: a well-conditioned stack converges on them; an ill-conditioned one (next to a
// Wood anomaly) stalls at that floor and only converges to 1e-9 on an FP64 residual, so its
// extra rounds take their products in FP64.  Products and sums follow Dekker / Knuth
// error-free transformations on the FP32 pipe, which on this GPU has ~60x the FP64 pipe's
// throughput; the rounded intrinsics keep the compiler from contracting the error terms.
__device__ __forceinline__ float4 df_of(cd v) {
  const float hr = (float)v.re, hi_ = (float)v.im;
  return make_float4(hr, hi_, (float)(v.re - (double)hr), (float)(v.im - (double)hi_));
}

__global__ void k_split_df(int64_t count, const cd* __restrict__ in, float4* __restrict__ out) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < count; e += (int64_t)gridDim.x * blockDim.x)
    out[e] = df_of(in[e]);
}

// (sh, sl) += (ah + al) (xh + xl), dropping al xl (relative 2^-48).
__device__ __forceinline__ void df_mac(float& sh, float& sl, float ah, float al, float xh, float xl) {
  const float p = __fmul_rn(ah, xh);
  float e = fmaf(ah, xh, -p);  // ah xh = p + e exactly
  e = fmaf(ah, xl, e);
  e = fmaf(al, xh, e);
  const float t = __fadd_rn(sh, p);  // two-sum: sh + p = t + err exactly
  const float bb = __fsub_rn(t, sh);
  const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, bb)), __fsub_rn(p, bb));
  sh = t;
  sl += err + e;
}

// y = A x for two columns, A row-major n x n as double-float pairs, x [n][2] as double-float
// pairs, y [n][2] FP64 (hi + lo of each accumulator).  A thread per row; x is read by every
// thread in the same order (broadcast loads).
__device__ void team_mv2_df(const TeamCta& t, const float4* __restrict__ A, int n, const float4* __restrict__ x,
                            cd* y) {
  for (int i = t.tid(); i < n; i += t.size()) {
    float r0h = 0.f, r0l = 0.f, i0h = 0.f, i0l = 0.f, r1h = 0.f, r1l = 0.f, i1h = 0.f, i1l = 0.f;
    const float4* row = A + (int64_t)i * n;
    for (int j = 0; j < n; ++j) {
      const float4 a = row[j];
      const float4 u = x[2 * j], v = x[2 * j + 1];
      // (a.x + i a.y) + (a.z + i a.w) times (u.x + i u.y) + (u.z + i u.w), column 0
      df_mac(r0h, r0l, a.x, a.z, u.x, u.z);
      df_mac(r0h, r0l, -a.y, -a.w, u.y, u.w);
      df_mac(i0h, i0l, a.x, a.z, u.y, u.w);
      df_mac(i0h, i0l, a.y, a.w, u.x, u.z);
      df_mac(r1h, r1l, a.x, a.z, v.x, v.z);
      df_mac(r1h, r1l, -a.y, -a.w, v.y, v.w);
      df_mac(i1h, i1l, a.x, a.z, v.y, v.w);
      df_mac(i1h, i1l, a.y, a.w, v.x, v.z);
    }
    y[2 * i] = mk((double)r0h + (double)r0l, (double)i0h + (double)i0l);
    y[2 * i + 1] = mk((double)r1h + (double)r1l, (double)i1h + (double)i1l);
  }
}

__global__ void k_round(int64_t count, const cd* __restrict__ in, cf* out) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < count; e += (int64_t)gridDim.x * blockDim.x)
    out[e] = mk((float)in[e].re, (float)in[e].im);
}

// ------------------------------------------------------------------------------------------
// Element table for the per-problem vector kernels
// ------------------------------------------------------------------------------------------
struct Elem {
  int kind;  // 0 homogeneous layer, 1 patterned layer
  int slot;  // map slot (patterned)
  DepthSel dep;
  const M2* blocks;  // homogeneous: [batch][nh][4] (FP64)
  const cf* inv1;  // homogeneous: M^-1; patterned: (F - G)^-1
  const cf* inv2;  // patterned: (P1 - P2)^-1
  const cf* zr;    // homogeneous: Gamma M^-1;  patterned: rho
};

struct MapPtrs {
  const cd* W64;
  const cd* V64;
  const cd* lam64;
  const cf* W32;
  const cf* V32;
  const cf* lam32;
  const cf* Wi;
  const cf* Vi;
  const float4* W2;  // W64 and V64 as double-float pairs {hi.re, hi.im, lo.re, lo.im} (k_split_df)
  const float4* V2;
};

struct Table {
  int L;
  int nh;
  int64_t batch;
  const M2* inc;
  const M2* trn;
  const cf* inv0;  // (I - S22_inc Gamma_0)^-1
  const cf* gam;   // Gamma at gaps 0..L: [L+1][batch][n][n]
  const M2* v0b;   // free-space V0 and V0^-1 blocks per problem and harmonic, [batch][nh]
  const M2* v0ib;
  Elem e[kMaxLayers];
  MapPtrs m[kMaxLayers];
};

// Unknowns of one problem (FP64), two columns each, [..][n][2]:
//   gap g = 0..L: c+ at x + (2g) * 2n, c- at x + (2g+1) * 2n;
//   patterned layer l: a+ at xa + (2l) * 2n, a- at xa + (2l+1) * 2n;   r, t.
// Residual slots per element (FP64): 4 x [n][2]; element 0 = incidence, 1..L layers, L+1 emergence.

template <typename V>
__device__ __forceinline__ cd ld2(const V* v, int i, int c) {
  return mk((double)v[2 * i + c].re, (double)v[2 * i + c].im);
}

// y = A x for two columns; A row-major n x n, x, y [n][2]; accumulation in A's precision.  A
// thread per row.  FP32 A with n even (n = 2 nh here): two elements per 16-byte load (row
// starts are 16-byte aligned since n is even and the matrices 256-byte aligned), which halves the
// L1 requests of these row-strided loads.
template <typename TA, typename TX, typename TY>
__device__ void team_mv2(const TeamCta& t, const cplx<TA>* A, int n, const cplx<TX>* x, cplx<TY>* y) {
  if constexpr (sizeof(TA) == 4) {
    if ((n & 1) == 0) {
      for (int i = t.tid(); i < n; i += t.size()) {
        cplx<TA> a0 = mk(TA(0)), a1 = mk(TA(0));
        const float4* row = reinterpret_cast<const float4*>(A + (int64_t)i * n);
        for (int j2 = 0; j2 < n / 2; ++j2) {
          const float4 v = row[j2];
          const int j = 2 * j2;
          const cplx<TA> p = mk(v.x, v.y), q = mk(v.z, v.w);
          fma_acc(a0, p, mk((TA)x[2 * j].re, (TA)x[2 * j].im));
          fma_acc(a1, p, mk((TA)x[2 * j + 1].re, (TA)x[2 * j + 1].im));
          fma_acc(a0, q, mk((TA)x[2 * j + 2].re, (TA)x[2 * j + 2].im));
          fma_acc(a1, q, mk((TA)x[2 * j + 3].re, (TA)x[2 * j + 3].im));
        }
        y[2 * i] = mk((TY)a0.re, (TY)a0.im);
        y[2 * i + 1] = mk((TY)a1.re, (TY)a1.im);
      }
      return;
    }
  }
  for (int i = t.tid(); i < n; i += t.size()) {
    cplx<TA> a0 = mk(TA(0)), a1 = mk(TA(0));
    const cplx<TA>* row = A + (int64_t)i * n;
    for (int j = 0; j < n; ++j) {
      const cplx<TA> aij = row[j];
      fma_acc(a0, aij, mk((TA)x[2 * j].re, (TA)x[2 * j].im));
      fma_acc(a1, aij, mk((TA)x[2 * j + 1].re, (TA)x[2 * j + 1].im));
    }
    y[2 * i] = mk((TY)a0.re, (TY)a0.im);
    y[2 * i + 1] = mk((TY)a1.re, (TY)a1.im);
  }
}

// y = S_q x for a per-harmonic block matrix (q = 0..3: S11, S12, S21, S22).
template <typename TX>
__device__ __forceinline__ cd blk_mv(const M2* S, int q, int nh, int i, int c, const TX* x) {
  const int g = i % nh, rb = i / nh;
  const M2& s = S[g * 4 + q];
  return blk(s, rb, 0) * ld2(x, g, c) + blk(s, rb, 1) * ld2(x, nh + g, c);
}

__device__ __forceinline__ cd src_col(const M2* S, int q, int nh, int i, int c) {
  const int g = i % nh;
  return g == (nh - 1) / 2 ? blk(S[g * 4 + q], i / nh, c) : mk(0.0);
}

__device__ __forceinline__ cd xprop(const cd* lam64, int i, double dk) { return cexp(-(lam64[i] * dk)); }

// FP64 residual of the stack equations at the current unknowns x (see the Elem comments).
__global__ void __launch_bounds__(256) k_stack_residual(Table tb, const double* gx, const double* gy,
                                                        const double* kp, const double* k0v, const cd* __restrict__ X,
                                                        const cd* __restrict__ XA, const cd* __restrict__ RT,
                                                        cd* RES, cd* scratch, const int* active, int x_zero,
                                                        int use_df) {
  TeamCta t;
  const int64_t b = blockIdx.x;
  if (active && !active[b]) return;
  if (x_zero) {
    // every unknown is zero (the first round): only the incidence source terms remain, and the
    // FP64 products of the layers would multiply zeros
    const int nh = tb.nh, n = 2 * nh, L = tb.L;
    const M2* S = tb.inc + b * nh * 4;
    cd* res = RES + b * (int64_t)(L + 2) * 4 * 2 * n;
    for (int64_t e = t.tid(); e < (int64_t)(L + 2) * 4 * 2 * n; e += t.size()) {
      const int i = (int)(e % (2 * n)) / 2, c = (int)(e % 2);
      res[e] = e < 2 * n ? src_col(S, 0, nh, i, c) : e < 4 * n ? src_col(S, 2, nh, i, c) : mk(0.0);
    }
    return;
  }
  const int nh = tb.nh, n = 2 * nh, L = tb.L;
  const int64_t nn = (int64_t)n * n;
  const int64_t xs = (int64_t)(2 * (L + 1)) * 2 * n, xas = (int64_t)2 * L * 2 * n;
  const cd* x = X + b * xs;
  const cd* xa = XA + b * xas;
  const cd* r = RT + b * 2 * n;
  const cd* tt = RT + (tb.batch + b) * 2 * n;
  cd* res = RES + b * (int64_t)(L + 2) * 4 * 2 * n;
  cd* w1 = scratch + b * 4 * 2 * n;
  cd* w2 = w1 + 2 * n;
  cd* w3 = w2 + 2 * n;
  cd* w4 = w3 + 2 * n;
  const double k0 = k0v[b];
  auto cp = [&](int g) { return x + (2 * g) * 2 * n; };
  auto cm = [&](int g) { return x + (2 * g + 1) * 2 * n; };
  // incidence: rA = S11 c + S12 c-_0 - r ; rB = S21 c + S22 c-_0 - c+_0
  {
    const M2* S = tb.inc + b * nh * 4;
    cd* rA = res;
    cd* rB = res + 2 * n;
    for (int e = t.tid(); e < 2 * n; e += t.size()) {
      const int i = e / 2, c = e % 2;
      rA[e] = src_col(S, 0, nh, i, c) + blk_mv(S, 1, nh, i, c, cm(0)) - r[e];
      rB[e] = src_col(S, 2, nh, i, c) + blk_mv(S, 3, nh, i, c, cm(0)) - cp(0)[e];
    }
  }
  int pl = 0;
  for (int l = 0; l < L; ++l) {
    const Elem& E = tb.e[l];
    cd* rs = res + (int64_t)(l + 1) * 4 * 2 * n;
    const cd *cpl = cp(l), *cml = cm(l), *cpr = cp(l + 1), *cmr = cm(l + 1);
    if (E.kind == 0) {
      const M2* S = E.blocks + b * nh * 4;
      for (int e = t.tid(); e < 2 * n; e += t.size()) {
        const int i = e / 2, c = e % 2;
        rs[e] = blk_mv(S, 0, nh, i, c, cpl) + blk_mv(S, 1, nh, i, c, cmr) - cml[e];
        rs[2 * n + e] = blk_mv(S, 2, nh, i, c, cpl) + blk_mv(S, 3, nh, i, c, cmr) - cpr[e];
      }
      t.sync();
      continue;
    }
    const MapPtrs& M = tb.m[E.slot];
    const cd* W = M.W64 + b * nn;
    const cd* V = M.V64 + b * nn;
    const cd* lam = M.lam64 + b * n;
    const double dk = E.dep.at(b) * k0;
    const cd* ap = xa + (2 * pl) * 2 * n;
    const cd* am = xa + (2 * pl + 1) * 2 * n;
    cd* r1 = rs;
    cd* r2 = rs + 2 * n;
    cd* r3 = rs + 4 * n;
    cd* r4 = rs + 6 * n;
    // w1 = a+ + X a-, w2 = X a- - a+, w3 = X a+ + a-, w4 = a- - X a+
    if (use_df && M.W2) {
      // the products W w, V w in double-float on the FP32 pipe (w1..w4 as pairs in the scratch)
      float4* f1 = reinterpret_cast<float4*>(w1);
      float4* f2 = f1 + 2 * n;
      float4* f3 = f2 + 2 * n;
      float4* f4 = f3 + 2 * n;
      for (int e = t.tid(); e < 2 * n; e += t.size()) {
        const cd xi = xprop(lam, e / 2, dk);
        f1[e] = df_of(ap[e] + xi * am[e]);
        f2[e] = df_of(xi * am[e] - ap[e]);
        f3[e] = df_of(xi * ap[e] + am[e]);
        f4[e] = df_of(am[e] - xi * ap[e]);
      }
      t.sync();
      const float4* W2 = M.W2 + b * nn;
      const float4* V2 = M.V2 + b * nn;
      team_mv2_df(t, W2, n, f1, r1);
      team_mv2_df(t, V2, n, f2, r2);
      team_mv2_df(t, W2, n, f3, r3);
      team_mv2_df(t, V2, n, f4, r4);
    } else {
      for (int e = t.tid(); e < 2 * n; e += t.size()) {
        const cd xi = xprop(lam, e / 2, dk);
        w1[e] = ap[e] + xi * am[e];
        w2[e] = xi * am[e] - ap[e];
        w3[e] = xi * ap[e] + am[e];
        w4[e] = am[e] - xi * ap[e];
      }
      t.sync();
      team_mv2(t, W, n, w1, r1);
      team_mv2(t, V, n, w2, r2);
      team_mv2(t, W, n, w3, r3);
      team_mv2(t, V, n, w4, r4);
    }
    t.sync();
    for (int e = t.tid(); e < 2 * n; e += t.size()) {
      const int i = e / 2, c = e % 2;
      const int g = i % nh, rb = i / nh;
      const M2 v0 = tb.v0b[b * nh + g];
      const cd dl0 = cml[2 * g + c] - cpl[2 * g + c], dl1 = cml[2 * (nh + g) + c] - cpl[2 * (nh + g) + c];
      const cd dr0 = cmr[2 * g + c] - cpr[2 * g + c], dr1 = cmr[2 * (nh + g) + c] - cpr[2 * (nh + g) + c];
      r1[e] = r1[e] - cpl[e] - cml[e];
      r2[e] = r2[e] - (blk(v0, rb, 0) * dl0 + blk(v0, rb, 1) * dl1);
      r3[e] = r3[e] - cpr[e] - cmr[e];
      r4[e] = r4[e] - (blk(v0, rb, 0) * dr0 + blk(v0, rb, 1) * dr1);
    }
    t.sync();
    ++pl;
  }
  // emergence: rA = S11 c+_L - c-_L ; rB = S21 c+_L - t
  {
    const M2* S = tb.trn + b * nh * 4;
    cd* rA = res + (int64_t)(L + 1) * 4 * 2 * n;
    cd* rB = rA + 2 * n;
    for (int e = t.tid(); e < 2 * n; e += t.size()) {
      const int i = e / 2, c = e % 2;
      rA[e] = blk_mv(S, 0, nh, i, c, cp(L)) - cm(L)[e];
      rB[e] = blk_mv(S, 2, nh, i, c, cp(L)) - tt[e];
    }
  }
}

// FP32 affine sweep: solves the stack equations for the residual RES (correction system) with
// the kept factors, and adds the correction to the FP64 unknowns.
// Per problem workspace (FP32, [..][n][2]): s at every gap (L+1), per layer 5 vectors, 6 temps.
__global__ void __launch_bounds__(256) k_stack_sweep(Table tb, const double* gx, const double* gy, const double* kp,
                                                     const double* k0v, const cd* __restrict__ RES, cd* X, cd* XA,
                                                     cd* RT, cf* WS, double* corr, const int* active) {
  __shared__ TeamShared sh;
  TeamCta t;
  if (active && !active[blockIdx.x]) return;
  double cmax = 0.0;  // largest |correction| of r and t (this thread)
  const int64_t b = blockIdx.x;
  const int nh = tb.nh, n = 2 * nh, L = tb.L;
  const int64_t nn = (int64_t)n * n;
  const int64_t xs = (int64_t)(2 * (L + 1)) * 2 * n, xas = (int64_t)2 * L * 2 * n;
  cd* x = X + b * xs;
  cd* xa = XA + b * xas;
  cd* r = RT + b * 2 * n;
  cd* tt = RT + (tb.batch + b) * 2 * n;
  const cd* res = RES + b * (int64_t)(L + 2) * 4 * 2 * n;
  const int64_t wsz = (int64_t)(L + 1 + 5 * L + 6) * 2 * n;
  cf* ws = WS + b * wsz;
  auto S_at = [&](int g) { return ws + (int64_t)g * 2 * n; };           // s at gap g
  auto LV = [&](int l, int k) { return ws + (int64_t)(L + 1 + 5 * l + k) * 2 * n; };  // per-layer vectors
  cf* T0 = ws + (int64_t)(L + 1 + 5 * L) * 2 * n;
  cf* T1 = T0 + 2 * n;
  cf* T2 = T1 + 2 * n;
  cf* T3 = T2 + 2 * n;
  cf* dcp = T3 + 2 * n;  // running correction of c+ (FP32)
  cf* dcm = dcp + 2 * n;
  const double k0 = k0v[b];
  auto rsl = [&](int elem, int k) { return res + (int64_t)elem * 4 * 2 * n + (int64_t)k * 2 * n; };
  auto gam = [&](int g) { return tb.gam + ((int64_t)g * tb.batch + b) * nn; };
  // ---- backward ----
  {
    const cd* rA = rsl(L + 1, 0);
    cf* s = S_at(L);
    for (int e = t.tid(); e < 2 * n; e += t.size()) s[e] = mk((float)rA[e].re, (float)rA[e].im);
  }
  t.sync();
  for (int l = L - 1; l >= 0; --l) {
    const Elem& E = tb.e[l];
    const cf* sj = S_at(l + 1);
    cf* sl = S_at(l);
    const cd* f1 = rsl(l + 1, 0);
    const cd* f2 = rsl(l + 1, 1);
    if (E.kind == 0) {
      const M2* S = E.blocks + b * nh * 4;
      cf* w = LV(l, 0);
      for (int e = t.tid(); e < 2 * n; e += t.size()) {
        const int i = e / 2, c = e % 2;
        const cd v = blk_mv(S, 3, nh, i, c, sj) + f2[e];
        w[e] = mk((float)v.re, (float)v.im);
      }
      t.sync();
      team_mv2(t, E.zr + b * nn, n, w, T0);  // Z w
      t.sync();
      for (int e = t.tid(); e < 2 * n; e += t.size()) T1[e] = T0[e] + sj[e];
      t.sync();
      for (int e = t.tid(); e < 2 * n; e += t.size()) {
        const int i = e / 2, c = e % 2;
        const cd v = blk_mv(S, 1, nh, i, c, T1) + f1[e];
        sl[e] = mk((float)v.re, (float)v.im);
      }
      t.sync();
      continue;
    }
    const MapPtrs& M = tb.m[E.slot];
    const cd* f3 = rsl(l + 1, 2);
    const cd* f4 = rsl(l + 1, 3);
    const double dk = E.dep.at(b) * k0;
    // T0 = f3 - s ; T1 = f4 - V0 s
    for (int e = t.tid(); e < 2 * n; e += t.size()) {
      const int i = e / 2, c = e % 2;
      const int g = i % nh, rb = i / nh;
      const M2 v0 = tb.v0b[b * nh + g];
      const cd v0s = blk(v0, rb, 0) * ld2(sj, g, c) + blk(v0, rb, 1) * ld2(sj, nh + g, c);
      const cd a = f3[e] - ld2(sj, i, c);
      const cd bb = f4[e] - v0s;
      T0[e] = mk((float)a.re, (float)a.im);
      T1[e] = mk((float)bb.re, (float)bb.im);
    }
    t.sync();
    cf* g3 = T2;
    cf* g4 = T3;
    team_mv2(t, M.Wi + b * nn, n, T0, g3);
    team_mv2(t, M.Vi + b * nn, n, T1, g4);
    t.sync();
    cf* q = LV(l, 0);  // g3 - g4
    for (int e = t.tid(); e < 2 * n; e += t.size()) {
      q[e] = g3[e] - g4[e];
      T1[e] = g3[e] + g4[e];
    }
    t.sync();
    cf* h = LV(l, 1);
    team_mv2(t, E.zr + b * nn, n, q, T0);  // rho q
    t.sync();
    const cf* lam = M.lam32 + b * n;
    for (int e = t.tid(); e < 2 * n; e += t.size()) {
      h[e] = mk(0.5f, 0.f) * (T0[e] - T1[e]);
      const cd xi = cexp(-(mk((double)lam[e / 2].re, (double)lam[e / 2].im) * dk));
      const cd xh = xi * ld2(h, e / 2, e % 2);
      T2[e] = mk((float)xh.re, (float)xh.im);  // X h
    }
    t.sync();
    team_mv2(t, M.W32 + b * nn, n, T2, T0);  // W X h
    team_mv2(t, M.V32 + b * nn, n, T2, T1);  // V X h
    t.sync();
    cf* k1 = LV(l, 2);
    cf* k2 = LV(l, 3);
    const cd* f1p = rsl(l + 1, 0);
    const cd* f2p = rsl(l + 1, 1);
    for (int e = t.tid(); e < 2 * n; e += t.size()) {
      const int i = e / 2, c = e % 2;
      const int g = i % nh, rb = i / nh;
      const M2 vi = tb.v0ib[b * nh + g];
      const cd a1 = ld2(T0, i, c) + f1p[e];
      const cd u0 = ld2(T1, g, c) + f2p[2 * g + c], u1 = ld2(T1, nh + g, c) + f2p[2 * (nh + g) + c];
      const cd a2 = blk(vi, rb, 0) * u0 + blk(vi, rb, 1) * u1;
      k1[e] = mk((float)a1.re, (float)a1.im);
      k2[e] = mk((float)a2.re, (float)a2.im);
    }
    t.sync();
    for (int e = t.tid(); e < 2 * n; e += t.size()) T3[e] = k2[e] - k1[e];
    t.sync();
    team_mv2(t, gam(l), n, T3, T0);  // Gamma_{left} (k2 - k1)
    t.sync();
    for (int e = t.tid(); e < 2 * n; e += t.size()) sl[e] = mk(0.5f, 0.f) * (T0[e] + k1[e] + k2[e]);
    t.sync();
  }
  // ---- incidence: c+_0 = M0^-1 (S22 s_0 + rB), c-_0 = Gamma_0 c+_0 + s_0, r += S12 c-_0 + rA ----
  {
    const M2* S = tb.inc + b * nh * 4;
    const cd* rA = rsl(0, 0);
    const cd* rB = rsl(0, 1);
    const cf* s0 = S_at(0);
    for (int e = t.tid(); e < 2 * n; e += t.size()) {
      const int i = e / 2, c = e % 2;
      const cd v = blk_mv(S, 3, nh, i, c, s0) + rB[e];
      dcp[e] = mk((float)v.re, (float)v.im);
    }
    t.sync();
    team_mv2(t, tb.inv0 + b * nn, n, dcp, T1);
    t.sync();
    for (int e = t.tid(); e < 2 * n; e += t.size()) dcp[e] = T1[e];
    t.sync();
    team_mv2(t, gam(0), n, dcp, T0);
    t.sync();
    for (int e = t.tid(); e < 2 * n; e += t.size()) dcm[e] = T0[e] + s0[e];
    t.sync();
    for (int e = t.tid(); e < 2 * n; e += t.size()) {
      const int i = e / 2, c = e % 2;
      const cd d = blk_mv(S, 1, nh, i, c, dcm) + rA[e];
      r[e] += d;
      const double m = cabs(d);
      cmax = m == m ? fmax(cmax, m) : INFINITY;
      x[e] += ld2(dcp, i, c);
      x[2 * n + e] += ld2(dcm, i, c);
    }
    t.sync();
  }
  // ---- forward ----
  int pl = 0;
  for (int l = 0; l < L; ++l) {
    const Elem& E = tb.e[l];
    const cf* sr = S_at(l + 1);
    if (E.kind == 0) {
      const M2* S = E.blocks + b * nh * 4;
      const cf* w = LV(l, 0);
      for (int e = t.tid(); e < 2 * n; e += t.size()) {
        const int i = e / 2, c = e % 2;
        const cd v = blk_mv(S, 2, nh, i, c, dcp) + ld2(w, i, c);
        T0[e] = mk((float)v.re, (float)v.im);
      }
      t.sync();
      team_mv2(t, E.inv1 + b * nn, n, T0, dcp);
      t.sync();
    } else {
      const MapPtrs& M = tb.m[E.slot];
      const cf* q = LV(l, 0);
      const cf* h = LV(l, 1);
      const cf* k1 = LV(l, 2);
      const cf* k2 = LV(l, 3);
      const double dk = E.dep.at(b) * k0;
      const cf* lam = M.lam32 + b * n;
      cd* ap = xa + (2 * pl) * 2 * n;
      cd* am = xa + (2 * pl + 1) * 2 * n;
      for (int e = t.tid(); e < 2 * n; e += t.size()) T3[e] = mk(2.f, 0.f) * dcp[e] - k1[e] + k2[e];
      t.sync();
      team_mv2(t, E.inv2 + b * nn, n, T3, T0);  // a+
      t.sync();
      for (int e = t.tid(); e < 2 * n; e += t.size()) {
        const cd xi = cexp(-(mk((double)lam[e / 2].re, (double)lam[e / 2].im) * dk));
        const cd xa_ = xi * ld2(T0, e / 2, e % 2);
        T1[e] = mk((float)xa_.re, (float)xa_.im);  // X a+
        const cd v = 2.0 * xa_ + ld2(q, e / 2, e % 2);
        T2[e] = mk((float)v.re, (float)v.im);
      }
      t.sync();
      team_mv2(t, E.inv1 + b * nn, n, T2, dcp);  // c+ right
      team_mv2(t, E.zr + b * nn, n, T1, T3);     // rho X a+
      t.sync();
      for (int e = t.tid(); e < 2 * n; e += t.size()) {
        ap[e] += ld2(T0, e / 2, e % 2);
        am[e] += ld2(T3, e / 2, e % 2) + ld2(h, e / 2, e % 2);
      }
      t.sync();
      ++pl;
    }
    // c-_{l+1} = Gamma c+ + s
    team_mv2(t, gam(l + 1), n, dcp, T0);
    t.sync();
    cd* cpg = x + (2 * (l + 1)) * 2 * n;
    cd* cmg = x + (2 * (l + 1) + 1) * 2 * n;
    for (int e = t.tid(); e < 2 * n; e += t.size()) {
      dcm[e] = T0[e] + sr[e];
      cpg[e] += ld2(dcp, e / 2, e % 2);
      cmg[e] += ld2(dcm, e / 2, e % 2);
    }
    t.sync();
  }
  // ---- emergence: t += S21 c+_L + rB ----
  {
    const M2* S = tb.trn + b * nh * 4;
    const cd* rB = rsl(L + 1, 1);
    for (int e = t.tid(); e < 2 * n; e += t.size()) {
      const int i = e / 2, c = e % 2;
      const cd d = blk_mv(S, 2, nh, i, c, dcp) + rB[e];
      tt[e] += d;
      const double m = cabs(d);
      cmax = m == m ? fmax(cmax, m) : INFINITY;
    }
  }
  int where = 0;
  team_argmax(t, cmax, where, &sh);
  if (t.tid() == 0) corr[b] = cmax;
}

// Convergence of the iterative refinement from the last two correction sizes: with linear
// convergence at rate c1 / c0 the remaining error is about c1^2 / (c0 - c1).  A problem stays
// active (needs more rounds) while its estimate exceeds 1e-9, its corrections do not shrink,
// or they are not finite; only problems already active are examined (null: all).
__global__ void k_check_refine(int64_t batch, const double* __restrict__ c0, const double* __restrict__ c1,
                               int* active) {
  for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < batch; b += (int64_t)gridDim.x * blockDim.x) {
    if (!active[b]) continue;
    const double a = c0[b], z = c1[b];
    const bool ok = z == 0.0 || (z < a && z * z <= 1e-9 * (a - z));
    active[b] = ok ? 0 : 1;
  }
}

__global__ void k_flag_unconverged(int64_t batch, const int* __restrict__ active, const double* __restrict__ kp,
                                   const double* __restrict__ k0, cd epsi, int* status) {
  for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < batch; b += (int64_t)gridDim.x * blockDim.x)
    if (active[b] && !rt_undefined(kp + 4 * b, k0[b], epsi)) status[b] |= KHP_BIT_REFINE;
}

#include "khp_adjoint.cuh"

// ------------------------------------------------------------------------------------------
// Gradient stage: per-problem M-bar^T = W H^T W^-1, then the convolution-matrix gradient.
// With N = M-bar^T (blocks N_ab, nh x nh), A1 = N21 Kx + N22 Ky, A2 = N11 Kx + N12 Ky
// (column scalings, normalised k), the transposed gradient of C for one problem is
//   A1 C^-1 Ky + A2 C^-1 Kx - N11 - N22 + QDT21 - QDT12 - C^-1 (Ky C A1 + Kx C A2) C^-1,
// from M = P Q with P, Q of alternative.py:158-178 (the diagonal-only terms cancel); QDT is
// the transposed direct term of Y = Q M^-1/2.  Sums over the problems that share a map are
// taken before the two products with C^-1 on the outside.
// ------------------------------------------------------------------------------------------
__global__ void k_make_a12(int64_t batch, int nh, const cf* __restrict__ N, const double* gx, const double* gy,
                           const double* kp, const double* k0, cf* A1, cf* A2) {
  const int n = 2 * nh;
  const int64_t hh = (int64_t)nh * nh, nn = (int64_t)n * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < batch * hh; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / hh;
    const int ij = (int)(e % hh);
    const int i = ij / nh, j = ij % nh;
    cd kx, ky;
    phys::kvec(kp, k0, gx, gy, b, j, kx, ky);
    const cf* Nb = N + b * nn;
    const cd n11 = to_d(Nb[(int64_t)i * n + j]), n12 = to_d(Nb[(int64_t)i * n + nh + j]);
    const cd n21 = to_d(Nb[(int64_t)(nh + i) * n + j]), n22 = to_d(Nb[(int64_t)(nh + i) * n + nh + j]);
    A1[e] = to_f(n21 * kx + n22 * ky);
    A2[e] = to_f(n11 * kx + n12 * ky);
  }
}

// E1 = G1 Ky + G2 Kx - N11 - N22 + QDT21 - QDT12 (column scalings), E2 = Ky G3 + Kx G4 (row
// scalings), with G1 = A1 C^-1, G2 = A2 C^-1, G3 = C A1, G4 = C A2.
__global__ void k_make_e12(int64_t batch, int nh, const cf* __restrict__ N, const cd* __restrict__ QDT,
                           const cf* __restrict__ G1, const cf* __restrict__ G2, const cf* __restrict__ G3,
                           const cf* __restrict__ G4, const double* gx, const double* gy, const double* kp,
                           const double* k0, cd* E1, cd* E2) {
  const int n = 2 * nh;
  const int64_t hh = (int64_t)nh * nh, nn = (int64_t)n * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < batch * hh; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / hh;
    const int ij = (int)(e % hh);
    const int i = ij / nh, j = ij % nh;
    cd kxj, kyj, kxi, kyi;
    phys::kvec(kp, k0, gx, gy, b, j, kxj, kyj);
    phys::kvec(kp, k0, gx, gy, b, i, kxi, kyi);
    const cf* Nb = N + b * nn;
    const cd* Qb = QDT + b * nn;
    const cd n11 = to_d(Nb[(int64_t)i * n + j]), n22 = to_d(Nb[(int64_t)(nh + i) * n + nh + j]);
    const cd q21 = Qb[(int64_t)(nh + i) * n + j], q12 = Qb[(int64_t)i * n + nh + j];
    E1[e] = to_d(G1[e]) * kyj + to_d(G2[e]) * kxj - n11 - n22 + q21 - q12;
    E2[e] = kyi * to_d(G3[e]) + kxi * to_d(G4[e]);
  }
}

// S[m] += sum of E[b] over the problems b with midx[b] == m (fixed order: deterministic).
__global__ void k_reduce_maps(int64_t batch, int64_t hh, int64_t nmaps, const int* __restrict__ midx,
                              const cd* __restrict__ E, cd* S) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nmaps * hh; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t m = e / hh, k = e % hh;
    cd acc = mk(0.0);
    for (int64_t b = 0; b < batch; ++b)
      if (midx[b] == m) acc += E[b * hh + k];
    S[e] += acc;
  }
}

// dconv[m][r][c] = -2 CT[m][c][r]: the gradient in the convention dL = Re sum(dconv o dC).
__global__ void k_dconv_out(int64_t nmaps, int nh, const cd* __restrict__ CT, cd* dconv) {
  const int64_t hh = (int64_t)nh * nh;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nmaps * hh; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t m = e / hh;
    const int rc = (int)(e % hh);
    const int r = rc / nh, c = rc % nh;
    dconv[e] = CT[m * hh + (int64_t)c * nh + r] * -2.0;
  }
}

struct GradArgs {
  const double* ic;  // C^-1 of every map, complex [nmaps][nh][nh]
  const double* wR;  // dL/dR per order, [batch][npol][nh] (null: 0)
  const double* wT;  // dL/dT per order
  double* Ro;        // per-order powers out, [batch][npol][nh] (null: not written)
  double* To;
  double* dconv;     // complex [nmaps][nh][nh] out
};

// ------------------------------------------------------------------------------------------
struct Arena {
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

struct MixedPlan {
  // per map slot
  std::vector<cf*> W32, V32, lam32, Wi, Vi, Q0, Vt;
  std::vector<cd*> W64, V64, lam64;
  // modes scratch
  cf *M32, *Z32, *E32, *lu32;
  cd *M64, *MW64, *CW64, *Ct64, *mu64, *mu64b;
  int *pair, *nearest;  // eigen-refinement clusters: label and rank of every column, [bm][n]
  int *csz, *memb;      // cluster size per column [bm][n]; members [bm][n][kClusterMax]
  // 3xTF32 recursion products: split A operands that stay fixed through the recursion (W^-1, Q0,
  // W, Vt of every slot), scratch splits of the varying A and of B, the tensor-core error flag
  float *tfAc, *tfA, *tfB;
  int* tferr;
  size_t tfa, tfb;  // elements per problem
  cf* xc;               // column of the cluster transform per column, [bm][n][kClusterMax]
  int* piv;
  std::vector<int*> midx;  // per map slot: the map index of every problem
  // the modes of all map slots run as one batch of S x batch matrices (slot-major): per-matrix
  // copies of kp, k0 and a per-matrix status
  double *kpx, *k0x;
  int* statx;
  M2 *v0b, *v0ib;  // free-space blocks per matrix of the modes batch ([batch][nh] first: per problem)
  cf* xv;          // [batch][n] propagator diagonal
  // per layer
  std::vector<cf*> inv1, inv2, zr;
  std::vector<M2*> blocks;
  M2 *inc, *trn;
  cf *gam, *F, *Gb, *P, *inv0;
  // vectors
  cd *X, *XA, *RT, *RES, *scr;
  cf* SW;
  double* corr;  // [2][batch]: correction sizes of the last two refinement rounds
  int* active;   // [batch]: refinement not yet converged
  OzakiWs oz;    // digit arrays of the FP64-accurate tensor-core products (M W and C W)
};

MixedPlan plan_mixed(Arena& a, int64_t batch, int nh, int L, const int* kinds, int nmaps_used) {
  const size_t n = 2 * (size_t)nh, nn = n * n;
  MixedPlan p;
  const size_t S = std::max(nmaps_used, 1);
  const size_t bm = S * batch;  // matrices of the modes stage
  // per-slot arrays are slices of one slot-major block each
  auto slices = [&](auto* base, size_t per, auto& vec) {
    for (int m = 0; m < nmaps_used; ++m) vec.push_back(base ? base + m * per : nullptr);
  };
  slices(a.take<cf>(bm * nn), batch * nn, p.W32);
  slices(a.take<cf>(bm * nn), batch * nn, p.V32);
  slices(a.take<cf>(bm * n), batch * n, p.lam32);
  slices(a.take<cf>(bm * nn), batch * nn, p.Wi);
  slices(a.take<cf>(bm * nn), batch * nn, p.Vi);
  slices(a.take<cf>(bm * nn), batch * nn, p.Q0);
  slices(a.take<cf>(bm * nn), batch * nn, p.Vt);
  slices(a.take<cd>(bm * nn), batch * nn, p.W64);
  slices(a.take<cd>(bm * nn), batch * nn, p.V64);
  slices(a.take<cd>(bm * n), batch * n, p.lam64);
  slices(a.take<int>(bm), batch, p.midx);
  p.M32 = a.take<cf>(bm * nn);
  p.Z32 = a.take<cf>(bm * nn);
  p.E32 = a.take<cf>(bm * nn);
  p.lu32 = a.take<cf>(bm * nn);
  // M64 and MW64 are one block: free while the eigensolver runs, it holds its rotation logs
  p.M64 = a.take<cd>(2 * bm * nn);
  p.MW64 = p.M64 ? p.M64 + bm * nn : nullptr;
  p.CW64 = a.take<cd>(bm * nn);
  p.Ct64 = nullptr;
  p.mu64 = a.take<cd>(bm * n);
  p.mu64b = a.take<cd>(bm * n);
  p.pair = a.take<int>(bm * n);
  p.nearest = a.take<int>(bm * n);
  p.csz = a.take<int>(bm * n);
  p.memb = a.take<int>(bm * n * kClusterMax);
  p.xc = a.take<cf>(bm * n * kClusterMax);
  p.piv = a.take<int>(bm * n);
  if (nmaps_used > 0) {
    // sized for M W (n x n x n); the C W products (nh x n, inner nh) need less
    const size_t ch = (size_t)ozaki_chunk((int64_t)bm);
    p.oz.ad_elems = ch * ozaki_a_elems((int)n, (int)n);
    p.oz.ad = a.take<uint16_t>(p.oz.ad_elems);
    p.oz.ea_n = ch * ozaki_rows_padded((int)n);
    p.oz.ea = a.take<int>(p.oz.ea_n);
    p.oz.bd_elems = ch * ozaki_b_elems((int)n, (int)n);
    p.oz.bd = a.take<uint16_t>(p.oz.bd_elems);
    p.oz.eb_n = ch * n;
    p.oz.eb = a.take<int>(p.oz.eb_n);
    p.oz.err = a.take<int>(1);
  }
  p.kpx = a.take<double>(bm * 4);
  p.k0x = a.take<double>(bm);
  p.statx = a.take<int>(bm);
  p.v0b = a.take<M2>(bm * nh);
  p.v0ib = a.take<M2>(bm * nh);
  p.xv = a.take<cf>(batch * n);
  for (int l = 0; l < L; ++l) {
    p.inv1.push_back(a.take<cf>(batch * nn));
    p.zr.push_back(a.take<cf>(batch * nn));
    if (kinds[l] == 1) {
      p.inv2.push_back(a.take<cf>(batch * nn));
      p.blocks.push_back(nullptr);
    } else {
      p.inv2.push_back(nullptr);
      p.blocks.push_back(a.take<M2>(batch * nh * 4));
    }
  }
  p.inc = a.take<M2>(batch * nh * 4);
  p.trn = a.take<M2>(batch * nh * 4);
  p.tfAc = p.tfA = p.tfB = nullptr;
  p.tferr = nullptr;
  p.tfa = p.tfb = 0;
  if (use_tf32_products((int)n)) {
    p.tfa = tf32x3_a_elems((int)n, (int)n);
    p.tfb = tf32x3_b_elems((int)n, (int)n);
    p.tfAc = a.take<float>((size_t)4 * S * batch * p.tfa);
    // the recursion's per-product planes, first used by the modes stage's S * batch products
    p.tfA = a.take<float>((size_t)S * batch * p.tfa);
    p.tfB = a.take<float>((size_t)S * batch * p.tfb);
    p.tferr = a.take<int>(1);
  }
  p.gam = a.take<cf>((size_t)(L + 1) * batch * nn);
  p.F = a.take<cf>(batch * nn);
  p.Gb = a.take<cf>(batch * nn);
  p.P = a.take<cf>(batch * nn);
  p.inv0 = a.take<cf>(batch * nn);
  p.X = a.take<cd>(batch * (size_t)(2 * (L + 1)) * 2 * n);
  p.XA = a.take<cd>(batch * (size_t)(2 * std::max(L, 1)) * 2 * n);
  p.RT = a.take<cd>(batch * 4 * n);
  p.RES = a.take<cd>(batch * (size_t)(L + 2) * 4 * 2 * n);
  p.scr = a.take<cd>(batch * 4 * 2 * n);
  p.SW = a.take<cf>(batch * (size_t)(L + 1 + 5 * L + 6) * 2 * n);
  p.corr = a.take<double>(2 * (size_t)batch);
  p.active = a.take<int>(batch);
  return p;
}

struct GradPlan {
  cd *Y, *RX, *RXA, *RRT, *GR, *GT, *scr4, *VEC, *HT, *QDT, *E1, *E2, *S1, *S2, *CT, *TMP;
  cf *SWT, *H32, *T32, *N32, *A1, *A2, *G1, *G2, *G3, *G4, *C32, *IC32;
};

GradPlan plan_grad(Arena& a, int64_t batch, int nh, int L, int64_t nmaps) {
  const size_t n = 2 * (size_t)nh, nn = n * n, hh = (size_t)nh * nh;
  GradPlan g;
  g.Y = a.take<cd>(batch * (size_t)(L + 2) * 4 * 2 * n);
  g.RX = a.take<cd>(batch * (size_t)(2 * (L + 1)) * 2 * n);
  g.RXA = a.take<cd>(batch * (size_t)(2 * std::max(L, 1)) * 2 * n);
  g.RRT = a.take<cd>(batch * 4 * n);
  g.GR = a.take<cd>(batch * 2 * n);
  g.GT = a.take<cd>(batch * 2 * n);
  g.scr4 = a.take<cd>(batch * 4 * 2 * n);
  g.VEC = a.take<cd>(batch * 20 * n);
  g.HT = a.take<cd>(batch * nn);
  g.QDT = a.take<cd>(batch * nn);
  g.E1 = a.take<cd>(batch * hh);
  g.E2 = a.take<cd>(batch * hh);
  g.S1 = a.take<cd>(nmaps * hh);
  g.S2 = a.take<cd>(nmaps * hh);
  g.CT = a.take<cd>(nmaps * hh);
  g.TMP = a.take<cd>(nmaps * hh);
  g.SWT = a.take<cf>(batch * (size_t)(L + 1 + 4 * L + 8) * 2 * n);
  g.H32 = a.take<cf>(batch * nn);
  g.T32 = a.take<cf>(batch * nn);
  g.N32 = a.take<cf>(batch * nn);
  g.A1 = a.take<cf>(batch * hh);
  g.A2 = a.take<cf>(batch * hh);
  g.G1 = a.take<cf>(batch * hh);
  g.G2 = a.take<cf>(batch * hh);
  g.G3 = a.take<cf>(batch * hh);
  g.G4 = a.take<cf>(batch * hh);
  g.C32 = a.take<cf>(nmaps * hh);
  g.IC32 = a.take<cf>(nmaps * hh);
  return g;
}

#define MX_TRY(x)        \
  do {                   \
    const int _s = (x);  \
    if (_s) return _s;   \
  } while (0)
#define MX_EW(kernel, total, ...)                                        \
  do {                                                                   \
    kernel<<<grid_for(total), 256, 0, s>>>(__VA_ARGS__);                 \
    count_launches(1);                                                   \
    MX_TRY(cuda_status());                                               \
  } while (0)

// A per-problem element-wise kernel (first parameter: the problem offset of the launch; one grid
// row per problem, per_problem_blocks(elems) CTAs along x), in launches of at most 65535 problems.
#define MX_PP(kernel, nprob, elems, ...)                                                               \
  do {                                                                                                 \
    for (int64_t _o = 0; _o < (int64_t)(nprob); _o += 65535) {                                         \
      const unsigned _nb = (unsigned)std::min<int64_t>((int64_t)(nprob) - _o, 65535);                  \
      kernel<<<dim3(per_problem_blocks(elems), _nb), 256, 0, s>>>(_o, __VA_ARGS__);                    \
      count_launches(1);                                                                               \
    }                                                                                                  \
    MX_TRY(cuda_status());                                                                             \
  } while (0)

// Backward stage of khp_solve_batched_mixed_grad (after the forward refinement): loss seeds,
// the adjoint solve (FP64 transposed residual + FP32 transposed sweep, refine + 3 rounds), the
// per-layer M-gradients and the convolution-matrix gradient of every map.
template <class DepthOf>
int grad_mixed(const Table& tb, MixedPlan& p, GradPlan& g, const GradArgs& ga, int64_t batch, int nh, int L,
               const int* kinds, const std::vector<int>& slot, const std::vector<int>& used, DepthOf depth_of,
               int64_t nmaps, const double* conv, const double* gx, const double* gy, const double* kp,
               const double* k0, int npol, const double* te, const double* tm, cd epsi, cd epse, int refine, double* R,
               double* Tt, const int* status, cudaStream_t s) {
  const int n = 2 * nh;
  const int64_t nn = (int64_t)n * n, hh = (int64_t)nh * nh;
  const cf one = mk(1.f), zero = mk(0.f);
  const cd done = mk(1.0), dzero = mk(0.0), dmone = mk(-1.0);
  k_flux_grad<<<(unsigned)batch, 128, 0, s>>>(nh, npol, p.RT, p.RT + batch * 2 * n, gx, gy, kp, k0,
                                              reinterpret_cast<const cd*>(te), reinterpret_cast<const cd*>(tm), epsi,
                                              epse, ga.wR, ga.wT, R, Tt, ga.Ro, ga.To, g.GR, g.GT);
  count_launches(1);
  MX_TRY(cuda_status());
  MX_EW(k_drop_unconverged_seeds, batch * 2 * n, batch, 2 * n, status, g.GR, g.GT);
  // ---- adjoint: F^T y = g ----
  if (cudaMemsetAsync(g.Y, 0, sizeof(cd) * batch * (size_t)(L + 2) * 4 * 2 * n, s) != cudaSuccess)
    return KHP_ERR_CUDA;
  for (int it = 0; it < refine + 3; ++it) {
    k_stack_residual_T<<<(unsigned)batch, 256, 0, s>>>(tb, gx, gy, kp, k0, g.Y, g.GR, g.GT, g.RX, g.RXA, g.RRT,
                                                       g.scr4);
    count_launches(1);
    MX_TRY(cuda_status());
    k_stack_sweep_T<<<(unsigned)batch, 256, 0, s>>>(tb, gx, gy, kp, k0, g.RX, g.RXA, g.RRT, g.Y, g.SWT);
    count_launches(1);
    MX_TRY(cuda_status());
  }
  // ---- per map slot: H^T, QD^T over its layers, then N = W H^T W^-1 and the C-gradient ----
  const cd* Cm = reinterpret_cast<const cd*>(conv);
  const cd* ICm = reinterpret_cast<const cd*>(ga.ic);
  MX_EW(k_round, nmaps * hh, nmaps * hh, Cm, g.C32);
  MX_EW(k_round, nmaps * hh, nmaps * hh, ICm, g.IC32);
  if (cudaMemsetAsync(g.S1, 0, sizeof(cd) * nmaps * hh, s) != cudaSuccess) return KHP_ERR_CUDA;
  if (cudaMemsetAsync(g.S2, 0, sizeof(cd) * nmaps * hh, s) != cudaSuccess) return KHP_ERR_CUDA;
  const int64_t ys_stride = (int64_t)(L + 2) * 4 * 2 * n;
  const int64_t xas = (int64_t)2 * std::max(L, 1) * 2 * n;
  for (size_t m = 0; m < used.size(); ++m) {
    if (cudaMemsetAsync(g.HT, 0, sizeof(cd) * batch * nn, s) != cudaSuccess) return KHP_ERR_CUDA;
    if (cudaMemsetAsync(g.QDT, 0, sizeof(cd) * batch * nn, s) != cudaSuccess) return KHP_ERR_CUDA;
    int pl = 0;
    for (int l = 0; l < L; ++l) {
      if (kinds[l] != 1) continue;
      if (slot[l] == (int)m) {
        k_layer_vectors<<<(unsigned)batch, 256, 0, s>>>(tb, l, pl, k0, p.XA, g.Y, g.VEC);
        count_launches(1);
        MX_TRY(cuda_status());
        MX_EW(k_layer_accum, batch * nn, batch, n, p.lam64[m], depth_of(l), k0, p.XA, xas, pl, g.Y, ys_stride,
              (int64_t)(l + 1) * 4 * 2 * n, g.VEC, g.HT, g.QDT);
      }
      ++pl;
    }
    MX_EW(k_round, batch * nn, batch * nn, g.HT, g.H32);
    MX_TRY(launch_gemm<float>(batch, n, n, n, one, p.W32[m], n, nn, g.H32, n, nn, zero, g.T32, n, nn, s));
    MX_TRY(launch_gemm<float>(batch, n, n, n, one, g.T32, n, nn, p.Wi[m], n, nn, zero, g.N32, n, nn, s));
    MX_EW(k_make_a12, batch * hh, batch, nh, g.N32, gx, gy, kp, k0, g.A1, g.A2);
    const int* mi = p.midx[m];
    MX_TRY(launch_gemm<float>(batch, nh, nh, nh, one, g.A1, nh, hh, g.IC32, nh, hh, zero, g.G1, nh, hh, s, nullptr,
                              mi));
    MX_TRY(launch_gemm<float>(batch, nh, nh, nh, one, g.A2, nh, hh, g.IC32, nh, hh, zero, g.G2, nh, hh, s, nullptr,
                              mi));
    MX_TRY(launch_gemm<float>(batch, nh, nh, nh, one, g.C32, nh, hh, g.A1, nh, hh, zero, g.G3, nh, hh, s, mi));
    MX_TRY(launch_gemm<float>(batch, nh, nh, nh, one, g.C32, nh, hh, g.A2, nh, hh, zero, g.G4, nh, hh, s, mi));
    MX_EW(k_make_e12, batch * hh, batch, nh, g.N32, g.QDT, g.G1, g.G2, g.G3, g.G4, gx, gy, kp, k0, g.E1, g.E2);
    MX_EW(k_reduce_maps, nmaps * hh, batch, hh, nmaps, mi, g.E1, g.S1);
    MX_EW(k_reduce_maps, nmaps * hh, batch, hh, nmaps, mi, g.E2, g.S2);
  }
  // ---- per map: CT = S1 - C^-1 S2 C^-1, dconv = -2 CT^T ----
  MX_TRY(launch_gemm<double>(nmaps, nh, nh, nh, done, g.S2, nh, hh, ICm, nh, hh, dzero, g.TMP, nh, hh, s));
  MX_TRY(launch_copy<double>(nmaps, nh, nh, g.S1, nh, hh, g.CT, nh, hh, s));
  MX_TRY(launch_gemm<double>(nmaps, nh, nh, nh, dmone, ICm, nh, hh, g.TMP, nh, hh, done, g.CT, nh, hh, s));
  MX_EW(k_dconv_out, nmaps * hh, nmaps, nh, g.CT, reinterpret_cast<cd*>(ga.dconv));
  return cuda_status();
}

int solve_mixed(int64_t batch, int px, int py, int L, const int* kinds, const int* maps, const double* eps,
                const double* depths, const int* pmap, const double* pdepth, int64_t nmaps, const double* conv,
                const double* hx, const double* hy, const double* gx,
                const double* gy, cd epsi, cd epse, const double* kp, const double* k0, int npol, const double* te,
                const double* tm, int refine, double* R, double* Tt, int* status, void* workspace, size_t ws_bytes,
                cudaStream_t s, const GradArgs* grad = nullptr) {
  const int nh = px * py, n = 2 * nh;
  const int64_t nn = (int64_t)n * n, hh = (int64_t)nh * nh, hn = (int64_t)nh * n;
  std::vector<int> used, first, slot(L, -1);
  for (int l = 0; l < L; ++l) {
    if (kinds[l] != 1) continue;
    int sidx = -1;
    for (size_t u = 0; u < used.size(); ++u)
      if (used[u] == maps[l]) sidx = (int)u;
    if (sidx < 0) {
      sidx = (int)used.size();
      used.push_back(maps[l]);
      first.push_back(l);
    }
    slot[l] = sidx;
  }
  auto depth_of = [&](int l) { return DepthSel{pdepth ? pdepth + (int64_t)l * batch : nullptr, depths[l]}; };
  Arena a{static_cast<char*>(workspace), ws_bytes};
  MixedPlan p = plan_mixed(a, batch, nh, L, kinds, (int)used.size());
  GradPlan gp{};
  if (grad) gp = plan_grad(a, batch, nh, L, nmaps);
  if (!a.ok || !workspace) return KHP_ERR_WORKSPACE;
  const cf one = mk(1.f), zero = mk(0.f), mone = mk(-1.f);
  const cd done = mk(1.0), dzero = mk(0.0);

  // ---- 1. modes: FP32 eigensolve + FP64 refinement, every map slot in one batch ----
  const int S = (int)used.size();
  if (S > 0) {
    stage_begin(KHP_STAGE_MODES, s);
    const int64_t bm = (int64_t)S * batch;
    const cd* Cm = reinterpret_cast<const cd*>(conv);
    const cd* HX = reinterpret_cast<const cd*>(hx);
    const cd* HY = reinterpret_cast<const cd*>(hy);
    int* const midx = p.midx[0];  // [S][batch]
    cf* const W32 = p.W32[0];
    cf* const V32 = p.V32[0];
    cf* const lam32 = p.lam32[0];
    cf* const Wi = p.Wi[0];
    cf* const Vi = p.Vi[0];
    cd* const W64 = p.W64[0];
    cd* const V64 = p.V64[0];
    cd* const lam64 = p.lam64[0];
    const double* kpx = p.kpx;
    const double* k0x = p.k0x;
    int* sx = p.statx;
    MX_EW(k_expand_problems, bm, bm, batch, S, kp, k0, p.kpx, p.k0x);
    if (cudaMemsetAsync(sx, 0, sizeof(int) * bm, s) != cudaSuccess) return KHP_ERR_CUDA;
    for (int m = 0; m < S; ++m)
      MX_EW(k_select_maps, batch, batch, pmap ? pmap + (int64_t)first[m] * batch : nullptr, used[m], nmaps,
            midx + (int64_t)m * batch, sx + (int64_t)m * batch);
    MX_TRY(launch_assemble_pq<float>(bm, nh, Cm, HX, HY, midx, gx, gy, kpx, k0x, p.M32, s));
    stage_begin(KHP_STAGE_EIGENSOLVE, s);
    MX_TRY(launch_geev<float>(bm, n, p.M32, n, nn, p.Z32, W32, n, nn, lam32, n, sx, s, p.M64,
                              (int64_t)(2 * nn * sizeof(cd))));
    stage_end(KHP_STAGE_EIGENSOLVE, s);
    // Refinement steps: R = M W - W mu in FP64, E = W^-1 R (FP32 inverse of the current W, held
    // in Wi until the final inverse), mu += diag(E), W += W F.
    MX_TRY(launch_assemble_pq<double>(bm, nh, Cm, HX, HY, midx, gx, gy, kpx, k0x, p.M64, s));
    MX_EW(k_to_double, bm * nn, bm * nn, W32, W64);
    MX_EW(k_to_double, bm * n, bm * n, lam32, p.mu64);
    MX_TRY(launch_copy<float>(bm, n, n, W32, n, nn, p.lu32, n, nn, s));
    MX_TRY(launch_inverse_blocked<float>(bm, n, p.lu32, n, nn, Wi, n, nn, p.piv, sx, s));
    cd* mu_a = p.mu64;
    cd* mu_b = p.mu64b;
    // the refinement steps' FP32 products (E = W^-1 R, W F): 3xTF32 on the tensor cores when the
    // recursion's products are (their planes are free until the recursion), else the tiled product
    auto mode_prod = [&](const cf* A, const cf* B, cf* C) -> int {
      if (!p.tfA) return launch_gemm<float>(bm, n, n, n, one, A, n, nn, B, n, nn, zero, C, n, nn, s);
      int st = tf32x3_split_a(bm, n, n, A, n, nn, nullptr, p.tfA, s);
      if (!st) st = tf32x3_split_b(bm, n, n, B, n, nn, nullptr, zero, p.tfB, s);
      return st ? st : tf32x3_from_planes(bm, n, n, n, p.tfA, p.tfB, one, zero, C, n, nn, p.tferr, s);
    };
    // M W in FP64 (tensor-core digit products) at every step.  Updating it in FP32 instead
    // (M W += round(M W) F) is only FP32-accurate where F is large: next to a nearly defective
    // cluster that error enters the next step's residual and the refinement stalls at ~1e-8.
    // (The structured product P (Q W) costs less but cancels terms of size k^4 / eps for the
    // evanescent orders.)
    for (int step = 0; step < kEigSteps; ++step) {
      if (step > 0) {
        // E with the inverse of the current W: the first step can rotate the vectors of a close
        // pair by ~1e-3, after which W0^-1 would make the later steps converge only linearly
        MX_TRY(launch_copy<float>(bm, n, n, W32, n, nn, p.lu32, n, nn, s));
        MX_TRY(launch_inverse_blocked<float>(bm, n, p.lu32, n, nn, Wi, n, nn, p.piv, sx, s));
      }
      MX_TRY(ozaki_zgemm(bm, n, n, n, p.M64, n, nn, nullptr, W64, n, nn, p.MW64, n, nn, p.oz, s,
                         mode_step_digits()));
      MX_PP(k_eig_residual, bm, nn, n, p.MW64, W64, mu_a, p.E32);
      MX_TRY(mode_prod(Wi, p.E32, p.Z32));  // E
      k_clusters<<<(unsigned)bm, 256, 0, s>>>(n, mu_a, p.Z32, p.pair, p.nearest, p.csz, p.memb, p.xc, mu_b);
      count_launches(1);
      MX_TRY(cuda_status());
      MX_PP(k_eig_update, bm, nn, n, mu_a, p.Z32, p.M32, p.pair, p.nearest, p.csz, p.memb, p.xc);  // M32 <- F
      MX_TRY(mode_prod(W32, p.M32, p.Z32));
      MX_EW(k_add_correction, bm * nn, bm * nn, W64, p.Z32, W32);
      std::swap(mu_a, mu_b);
    }
    // FP64 eigen-residual of the refined modes (KHP_BIT_MODES where a column missed 1e-8)
    MX_TRY(ozaki_zgemm(bm, n, n, n, p.M64, n, nn, nullptr, W64, n, nn, p.MW64, n, nn, p.oz, s));
    k_eig_check<<<(unsigned)bm, 256, 0, s>>>(n, p.MW64, W64, mu_a, kpx, k0x, epsi, sx);
    count_launches(1);
    MX_TRY(cuda_status());
    MX_EW(k_sqrt_mu, bm * n, bm * n, mu_a, lam64, lam32);
    // V = Q W / lam in FP64
    cd* CWt = p.CW64;
    cd* CWb = p.CW64 + hn;
    MX_TRY(ozaki_zgemm(bm, nh, n, nh, Cm, nh, hh, midx, W64, n, nn, CWt, n, nn, p.oz, s));
    MX_TRY(ozaki_zgemm(bm, nh, n, nh, Cm, nh, hh, midx, W64 + hn, n, nn, CWb, n, nn, p.oz, s));
    MX_TRY(launch_modes_v<double>(bm, nh, gx, gy, kpx, k0x, W64, CWt, CWb, nn, lam64, V64, sx, s));
    MX_EW(k_round, bm * nn, bm * nn, V64, V32);
    // W and V as double-float pairs for the stack residual, in the M, M W block (free from here on)
    MX_EW(k_split_df, bm * nn, bm * nn, W64, reinterpret_cast<float4*>(p.M64));
    MX_EW(k_split_df, bm * nn, bm * nn, V64, reinterpret_cast<float4*>(p.MW64));
    // FP32 inverses and V0 products
    MX_TRY(launch_copy<float>(bm, n, n, W32, n, nn, p.lu32, n, nn, s));
    MX_TRY(launch_inverse_blocked<float>(bm, n, p.lu32, n, nn, Wi, n, nn, p.piv, sx, s));
    MX_TRY(launch_copy<float>(bm, n, n, V32, n, nn, p.lu32, n, nn, s));
    MX_TRY(launch_inverse_blocked<float>(bm, n, p.lu32, n, nn, Vi, n, nn, p.piv, sx, s));
    MX_EW(k_v0_blocks, bm * nh, bm, nh, gx, gy, kpx, k0x, p.v0b, p.v0ib);
    MX_EW(k_v0_right<float>, bm * nn, bm, nh, p.v0b, Vi, p.Q0[0]);
    MX_EW(k_v0inv_left<float>, bm * nn, bm, nh, p.v0ib, V32, p.Vt[0]);
    MX_EW(k_or_status, batch, batch, S, sx, status);
    stage_end(KHP_STAGE_MODES, s);
  } else {
    MX_EW(k_v0_blocks, batch * nh, batch, nh, gx, gy, kp, k0, p.v0b, p.v0ib);
  }
  // ---- homogeneous blocks (FP64) ----
  stage_begin(KHP_STAGE_RECURSION, s);
  MX_EW(k_homog_blocks, batch * nh, batch, nh, 1, epsi, DepthSel{nullptr, 0.0}, gx, gy, kp, k0, p.inc, status);
  MX_EW(k_homog_blocks, batch * nh, batch, nh, 2, epse, DepthSel{nullptr, 0.0}, gx, gy, kp, k0, p.trn, status);
  for (int l = 0; l < L; ++l)
    if (kinds[l] != 1)
      MX_EW(k_homog_blocks, batch * nh, batch, nh, 0, mk(eps[2 * l], eps[2 * l + 1]), depth_of(l), gx, gy, kp, k0,
            p.blocks[l], status);
  // ---- 2. FP32 backward recursion, keeping every factor (explicit inverses: every O(n^3) step
  //         is then a blocked factorisation or a tiled product) ----
  auto gam = [&](int g) { return p.gam + (int64_t)g * batch * nn; };
  // The recursion's n x n FP32 products: 3xTF32 on the tensor cores (the split of every fixed A
  // operand made once per call), or the FP32 tiled product.  C = A (B + shift I).
  const bool tf = p.tfAc != nullptr;
  auto fixed_a = [&](int which, int m) { return p.tfAc + ((size_t)which * S + m) * batch * p.tfa; };
  if (tf) {
    for (int m = 0; m < S; ++m) {
      MX_TRY(tf32x3_split_a(batch, n, n, p.Wi[m], n, nn, nullptr, fixed_a(0, m), s));
      MX_TRY(tf32x3_split_a(batch, n, n, p.Q0[m], n, nn, nullptr, fixed_a(1, m), s));
      MX_TRY(tf32x3_split_a(batch, n, n, p.W32[m], n, nn, nullptr, fixed_a(2, m), s));
      MX_TRY(tf32x3_split_a(batch, n, n, p.Vt[m], n, nn, nullptr, fixed_a(3, m), s));
    }
  }
  auto prod_fixed = [&](int which, int m, const cf* A, const cf* B, cf shift, cf* C) -> int {
    if (!tf) return launch_gemm<float>(batch, n, n, n, one, A, n, nn, B, n, nn, zero, C, n, nn, s, nullptr, nullptr,
                                       shift);
    const int st = tf32x3_split_b(batch, n, n, B, n, nn, nullptr, shift, p.tfB, s);
    return st ? st : tf32x3_from_planes(batch, n, n, n, fixed_a(which, m), p.tfB, one, zero, C, n, nn, p.tferr, s);
  };
  auto prod = [&](const cf* A, const cf* B, cf* C) -> int {
    if (!tf) return launch_gemm<float>(batch, n, n, n, one, A, n, nn, B, n, nn, zero, C, n, nn, s);
    int st = tf32x3_split_a(batch, n, n, A, n, nn, nullptr, p.tfA, s);
    if (!st) st = tf32x3_split_b(batch, n, n, B, n, nn, nullptr, zero, p.tfB, s);
    return st ? st : tf32x3_from_planes(batch, n, n, n, p.tfA, p.tfB, one, zero, C, n, nn, p.tferr, s);
  };
  MX_EW(k_gamma_from_blocks<float>, batch * nn, batch, nh, p.trn, 0, gam(L));
  for (int l = L - 1; l >= 0; --l) {
    cf* G = gam(l + 1);
    if (kinds[l] != 1) {
      MX_TRY(launch_i_minus_sg<float>(batch, nh, p.blocks[l], G, p.lu32, s));
      MX_TRY(launch_inverse_blocked<float>(batch, n, p.lu32, n, nn, p.inv1[l], n, nn, p.piv, status, s));
      MX_TRY(prod(G, p.inv1[l], p.zr[l]));
      MX_TRY(launch_sandwich<float>(batch, nh, p.blocks[l], p.zr[l], gam(l), s));
    } else {
      const int m = slot[l];
      // F = Wi (G + I), Gb = Q0 (G - I): the identity added to G's diagonal as it is read
      MX_TRY(prod_fixed(0, m, p.Wi[m], G, one, p.F));
      MX_TRY(prod_fixed(1, m, p.Q0[m], G, mone, p.Gb));
      MX_EW(k_diff_sum<float>, batch * nn, batch * nn, p.F, p.Gb, p.lu32);
      MX_TRY(launch_inverse_blocked<float>(batch, n, p.lu32, n, nn, p.inv1[l], n, nn, p.piv, status, s));
      MX_TRY(prod(p.F, p.inv1[l], p.zr[l]));  // rho
      MX_TRY(launch_copy<float>(batch, n, n, p.zr[l], n, nn, p.F, n, nn, s));
      MX_EW(k_xvec<float>, batch * n, batch, n, p.lam32[m], depth_of(l), k0, p.xv);
      MX_EW(k_xmx_t<float>, batch * nn, batch, n, p.xv, p.F);
      // Gb = W (F + I), P = Vt (F - I)
      MX_TRY(prod_fixed(2, m, p.W32[m], p.F, one, p.Gb));
      MX_TRY(prod_fixed(3, m, p.Vt[m], p.F, mone, p.P));
      MX_EW(k_diff_sum<float>, batch * nn, batch * nn, p.Gb, p.P, p.lu32);
      MX_TRY(launch_inverse_blocked<float>(batch, n, p.lu32, n, nn, p.inv2[l], n, nn, p.piv, status, s));
      MX_TRY(prod(p.Gb, p.inv2[l], gam(l)));
    }
  }
  MX_TRY(launch_i_minus_sg<float>(batch, nh, p.inc, gam(0), p.lu32, s));
  MX_TRY(launch_inverse_blocked<float>(batch, n, p.lu32, n, nn, p.inv0, n, nn, p.piv, status, s));
  stage_end(KHP_STAGE_RECURSION, s);
  // ---- 3. iterative refinement of the stack equations ----
  stage_begin(KHP_STAGE_REFINE, s);
  Table tb;
  tb.L = L;
  tb.nh = nh;
  tb.batch = batch;
  tb.inc = p.inc;
  tb.trn = p.trn;
  tb.inv0 = p.inv0;
  tb.gam = p.gam;
  tb.v0b = p.v0b;
  tb.v0ib = p.v0ib;
  for (int l = 0; l < L; ++l) {
    Elem& E = tb.e[l];
    E.kind = kinds[l] == 1 ? 1 : 0;
    E.slot = slot[l];
    E.dep = depth_of(l);
    E.blocks = p.blocks[l];
    E.inv1 = p.inv1[l];
    E.inv2 = p.inv2[l];
    E.zr = p.zr[l];
  }
  for (size_t m = 0; m < used.size(); ++m) {
    MapPtrs& M = tb.m[m];
    M.W64 = p.W64[m];
    M.V64 = p.V64[m];
    M.lam64 = p.lam64[m];
    M.W32 = p.W32[m];
    M.V32 = p.V32[m];
    M.lam32 = p.lam32[m];
    M.Wi = p.Wi[m];
    M.Vi = p.Vi[m];
    M.W2 = p.M64 ? reinterpret_cast<const float4*>(p.M64) + m * (size_t)batch * nn : nullptr;
    M.V2 = p.MW64 ? reinterpret_cast<const float4*>(p.MW64) + m * (size_t)batch * nn : nullptr;
  }
  const size_t xbytes = sizeof(cd) * batch * (size_t)(2 * (L + 1)) * 2 * n;
  if (cudaMemsetAsync(p.X, 0, xbytes, s) != cudaSuccess) return KHP_ERR_CUDA;
  if (cudaMemsetAsync(p.XA, 0, sizeof(cd) * batch * (size_t)(2 * std::max(L, 1)) * 2 * n, s) != cudaSuccess)
    return KHP_ERR_CUDA;
  if (cudaMemsetAsync(p.RT, 0, sizeof(cd) * batch * 4 * n, s) != cudaSuccess) return KHP_ERR_CUDA;
  // refine rounds for every problem, then up to kExtraRounds more for the problems whose
  // estimated error is still above 1e-9 (the others skip them); problems still unconverged get
  // status bit 8.
  const int total = refine >= 1 ? refine + kExtraRounds : 0;
  for (int it = 0; it <= total; ++it) {
    const int* act = it > refine ? p.active : nullptr;
    // the refine rounds every problem runs take the products in double-float; the extra rounds
    // of the problems that have not converged by then (an ill-conditioned stack next to a Wood
    // anomaly, whose corrections stall at the double-float floor) take them in FP64
    k_stack_residual<<<(unsigned)batch, 256, 0, s>>>(tb, gx, gy, kp, k0, p.X, p.XA, p.RT, p.RES, p.scr, act,
                                                      it == 0 ? 1 : 0, it <= refine ? 1 : 0);
    count_launches(1);
    MX_TRY(cuda_status());
    k_stack_sweep<<<(unsigned)batch, 256, 0, s>>>(tb, gx, gy, kp, k0, p.RES, p.X, p.XA, p.RT, p.SW,
                                                   p.corr + (it & 1) * batch, act);
    count_launches(1);
    MX_TRY(cuda_status());
    if (it == refine && refine >= 1) {
      if (cudaMemsetAsync(p.active, 0xff, sizeof(int) * batch, s) != cudaSuccess) return KHP_ERR_CUDA;
    }
    if (it >= refine && refine >= 1)
      MX_EW(k_check_refine, batch, batch, p.corr + ((it - 1) & 1) * batch, p.corr + (it & 1) * batch, p.active);
  }
  if (refine >= 1) MX_EW(k_flag_unconverged, batch, batch, p.active, kp, k0, epsi, status);
  if (!grad) {
    k_flux_cols<double><<<(unsigned)batch, 128, 0, s>>>(nh, npol, p.RT, p.RT + batch * 2 * n, gx, gy, kp, k0,
                                                         reinterpret_cast<const cd*>(te),
                                                         reinterpret_cast<const cd*>(tm), epsi, epse, R, Tt);
    count_launches(1);
    stage_end(KHP_STAGE_REFINE, s);
    return cuda_status();
  }
  stage_end(KHP_STAGE_REFINE, s);
  return grad_mixed(tb, p, gp, *grad, batch, nh, L, kinds, slot, used, depth_of, nmaps, conv, gx, gy, kp, k0, npol,
                    te, tm, epsi, epse, refine, R, Tt, status, s);
}

}  // namespace

int mixed_modes_in_workspace(int64_t batch, int nh, int L, const int* kinds, const int* maps, const void* ws,
                             size_t ws_bytes, const cd** W, const cd** V, const cd** lam) {
  std::vector<int> used;
  for (int l = 0; l < L; ++l)
    if (kinds[l] == 1 && std::find(used.begin(), used.end(), maps[l]) == used.end()) used.push_back(maps[l]);
  *W = *V = *lam = nullptr;
  if (used.empty()) return KHP_OK;
  Arena a{static_cast<char*>(const_cast<void*>(ws)), ws_bytes};
  MixedPlan p = plan_mixed(a, batch, nh, L, kinds, (int)used.size());
  if (!a.ok || !ws) return KHP_ERR_WORKSPACE;
  *W = p.W64[0];
  *V = p.V64[0];
  *lam = p.lam64[0];
  return KHP_OK;
}

}  // namespace khp

using namespace khp;

extern "C" {

size_t khp_solve_batched_mixed_workspace(int64_t batch, int32_t nh, int32_t nlayers, const int32_t* layer_kind,
                                         const int32_t* layer_map) {
  if (batch < 0 || nh < 1 || nlayers < 0 || nlayers > kMaxLayers || (nlayers > 0 && (!layer_kind || !layer_map)))
    return 0;
  std::vector<int> seen;
  for (int l = 0; l < nlayers; ++l) {
    if (layer_kind[l] != 1) continue;
    if (std::find(seen.begin(), seen.end(), layer_map[l]) == seen.end()) seen.push_back(layer_map[l]);
  }
  Arena a{nullptr, 0};
  plan_mixed(a, batch, nh, nlayers, layer_kind, (int)seen.size());
  return a.off;
}

int khp_solve_batched_mixed(int64_t batch, int32_t px, int32_t py, int32_t nlayers, const int32_t* layer_kind,
                            const int32_t* layer_map, const double* layer_eps, const double* layer_depth,
                            const int32_t* problem_map, const double* problem_depth, int64_t nmaps,
                            const double* conv, const double* hx, const double* hy, const double* gx,
                            const double* gy, double epsi_re, double epsi_im, double epse_re, double epse_im,
                            const double* kp, const double* k0, int32_t npol, const double* te, const double* tm,
                            int32_t refine_iters, double* R, double* T, int32_t* status, void* workspace,
                            size_t ws_bytes, void* stream) {
  if (batch < 0 || px < 1 || py < 1 || nlayers < 0 || npol < 1 || refine_iters < 0 || refine_iters > kMaxRefine ||
      !gx || !gy || !kp || !k0 || !te || !tm || !R || !T || !status)
    return KHP_ERR_INVALID_ARG;
  if (nlayers > kMaxLayers) return KHP_ERR_TOO_LARGE;
  if (nlayers > 0 && (!layer_kind || !layer_map || !layer_eps || !layer_depth)) return KHP_ERR_INVALID_ARG;
  for (int l = 0; l < nlayers; ++l) {
    if (layer_kind[l] != 0 && layer_kind[l] != 1) return KHP_ERR_INVALID_ARG;
    if (layer_kind[l] == 1 && (layer_map[l] < 0 || layer_map[l] >= nmaps || !conv || !hx || !hy))
      return KHP_ERR_INVALID_ARG;
  }
  if (batch == 0) return KHP_OK;
  return solve_mixed(batch, px, py, nlayers, layer_kind, layer_map, layer_eps, layer_depth, problem_map,
                     problem_depth, nmaps, conv, hx, hy, gx, gy,
                     mk(epsi_re, epsi_im), mk(epse_re, epse_im), kp, k0, npol, te, tm, refine_iters, R, T, status,
                     workspace, ws_bytes, reinterpret_cast<cudaStream_t>(stream));
}

size_t khp_solve_batched_mixed_grad_workspace(int64_t batch, int32_t nh, int32_t nlayers, const int32_t* layer_kind,
                                              const int32_t* layer_map, int64_t nmaps) {
  const size_t fwd = khp_solve_batched_mixed_workspace(batch, nh, nlayers, layer_kind, layer_map);
  if (fwd == 0 || nmaps < 1) return 0;
  Arena a{nullptr, 0};
  a.off = fwd;
  plan_grad(a, batch, nh, nlayers, nmaps);
  return a.off;
}

int khp_solve_batched_mixed_grad(int64_t batch, int32_t px, int32_t py, int32_t nlayers, const int32_t* layer_kind,
                                 const int32_t* layer_map, const double* layer_eps, const double* layer_depth,
                                 const int32_t* problem_map, const double* problem_depth, int64_t nmaps,
                                 const double* conv, const double* ic, const double* hx, const double* hy,
                                 const double* gx, const double* gy, double epsi_re, double epsi_im, double epse_re,
                                 double epse_im, const double* kp, const double* k0, int32_t npol, const double* te,
                                 const double* tm, int32_t refine_iters, const double* dR, const double* dT, double* R,
                                 double* T, double* R_orders, double* T_orders, double* dconv, int32_t* status,
                                 void* workspace, size_t ws_bytes, void* stream) {
  if (batch < 0 || px < 1 || py < 1 || nlayers < 0 || npol < 1 || refine_iters < 1 || refine_iters > kMaxRefine ||
      !gx || !gy || !kp || !k0 || !te || !tm || !R || !T || !status || !dconv || !ic || nmaps < 1)
    return KHP_ERR_INVALID_ARG;
  if (nlayers > kMaxLayers) return KHP_ERR_TOO_LARGE;
  if (nlayers > 0 && (!layer_kind || !layer_map || !layer_eps || !layer_depth)) return KHP_ERR_INVALID_ARG;
  for (int l = 0; l < nlayers; ++l) {
    if (layer_kind[l] != 0 && layer_kind[l] != 1) return KHP_ERR_INVALID_ARG;
    if (layer_kind[l] == 1 && (layer_map[l] < 0 || layer_map[l] >= nmaps || !conv || !hx || !hy))
      return KHP_ERR_INVALID_ARG;
  }
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const int64_t hh = (int64_t)px * py * px * py;
  if (cudaMemsetAsync(dconv, 0, sizeof(double) * 2 * nmaps * hh, s) != cudaSuccess) return KHP_ERR_CUDA;
  if (batch == 0) return KHP_OK;
  GradArgs ga{ic, dR, dT, R_orders, T_orders, dconv};
  return solve_mixed(batch, px, py, nlayers, layer_kind, layer_map, layer_eps, layer_depth, problem_map,
                     problem_depth, nmaps, conv, hx, hy, gx, gy, mk(epsi_re, epsi_im), mk(epse_re, epse_im), kp, k0,
                     npol, te, tm, refine_iters, R, T, status, workspace, ws_bytes, s, &ga);
}

}  // extern "C"
