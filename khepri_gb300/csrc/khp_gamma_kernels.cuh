// Kernels of the batched reflection-matrix recursion (khp_solve_batched, khp_solve_batched_mixed):
// mode assembly and post-processing, free-space V0 products, closed-form homogeneous blocks,
// the per-harmonic structured products of the recursion, and the two-column flux.
// Templated on the storage type T of the dense matrices; per-harmonic physics in FP64.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>

#include "khp_dense.cuh"
#include "khp_launch.h"
#include "khp_physics.cuh"

namespace khp {
namespace {

using cd = cplx<double>;
using phys::M2;

// Per-problem depth of a layer: p[b] when the caller gave per-problem depths, else `fixed`.
struct DepthSel {
  const double* p;
  double fixed;
  __device__ __forceinline__ double at(int64_t b) const { return p ? p[b] : fixed; }
};

// Map index of every problem for one map slot: pm[b] from the caller's per-problem map table
// (column of the slot's first layer) or `fixed`; an index outside [0, nmaps) is replaced by 0
// and flags the problem (KHP_BIT_BAD_INPUT), so that no later kernel reads outside the maps.
__global__ void k_select_maps(int64_t batch, const int* __restrict__ pm, int fixed, int64_t nmaps, int* out,
                              int* status) {
  for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < batch; b += (int64_t)gridDim.x * blockDim.x) {
    const int m = pm ? pm[b] : fixed;
    const bool ok = m >= 0 && m < nmaps;
    out[b] = ok ? m : 0;
    if (!ok) atomicOr(status + b, KHP_BIT_BAD_INPUT);
  }
}

inline int grid_for(int64_t total) { return (int)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, 152 * 32)); }

template <typename T>
__device__ __forceinline__ cplx<T> to_t(cd z) { return mk((T)z.re, (T)z.im); }
template <typename T>
__device__ __forceinline__ cd to_d(cplx<T> z) { return mk((double)z.re, (double)z.im); }

// Element (r, c) of a 2x2 block: r, c in {0, 1}.
__device__ __forceinline__ cd blk(const M2& m, int r, int c) { return r == 0 ? (c == 0 ? m.a : m.b) : (c == 0 ? m.c : m.d); }

template <typename T>
__global__ void __launch_bounds__(256) k_getrs_right(int n, const cplx<T>* A, int64_t lda, int64_t bsA, const int* piv,
                                                      cplx<T>* B, int64_t ldb, int64_t bsB, int m) {
  TeamCta t;
  const int64_t b = blockIdx.x;
  team_getrs_right(t, A + b * bsA, lda, n, piv + b * n, B + b * bsB, ldb, m);
}

template <typename T>
__global__ void k_convert(int64_t count, const cd* __restrict__ in, cplx<T>* out) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < count; e += (int64_t)gridDim.x * blockDim.x)
    out[e] = to_t<T>(in[e]);
}

// M = P Q of one pixmap for every problem (same identity as khp_layer_modes); problem b uses
// map midx[b] of the [nmaps][nh][nh] arrays C, Hx, Hy.
// One grid row per problem (b = boff + blockIdx.y): the problem's per-harmonic wave vectors are
// tabulated in shared memory first (dynamic, 2 nh complex), so no element divides.  Launched by
// launch_assemble_pq.
template <typename T>
__global__ void k_assemble_pq_t(int64_t boff, int nh, const cd* __restrict__ Cm, const cd* __restrict__ Hxm,
                                const cd* __restrict__ Hym, const int* __restrict__ midx, const double* gx,
                                const double* gy, const double* kp, const double* k0, cplx<T>* M) {
  extern __shared__ cd kt_pq[];
  cd* kxs = kt_pq;
  cd* kys = kt_pq + nh;
  const int64_t b = boff + blockIdx.y;
  for (int g = threadIdx.x; g < nh; g += blockDim.x) phys::kvec(kp, k0, gx, gy, b, g, kxs[g], kys[g]);
  __syncthreads();
  const int n = 2 * nh, nn = n * n;
  const int64_t moff = (int64_t)midx[b] * nh * nh;
  const cd* C = Cm + moff;
  const cd* Hx = Hxm + moff;
  const cd* Hy = Hym + moff;
  const double k = k0[b], ik = 1.0 / k;
  const cd ax = mk(kp[4 * b + 0] / k, kp[4 * b + 1] / k), ay = mk(kp[4 * b + 2] / k, kp[4 * b + 3] / k);
  cplx<T>* Mb = M + b * (int64_t)nn;
  for (int rc = blockIdx.x * blockDim.x + threadIdx.x; rc < nn; rc += gridDim.x * blockDim.x) {
    const int r = rc / n, c = rc - r * n;
    const int bi = r >= nh ? 1 : 0, bj = c >= nh ? 1 : 0;
    const int i = r - bi * nh, j = c - bj * nh;
    const int64_t mo = (int64_t)i * nh + j;
    const cd kxi = kxs[i], kyi = kys[i];
    const bool dg = (i == j);
    const cd gxv = Hx[mo] * ik + (dg ? ax : mk(0.0));
    const cd gyv = Hy[mo] * ik + (dg ? ay : mk(0.0));
    cd v;
    if (bi == 0 && bj == 0) v = kxi * gxv - C[mo] + (dg ? kyi * kyi : mk(0.0));
    else if (bi == 0) v = kxi * gyv - (dg ? kxi * kyi : mk(0.0));
    else if (bj == 0) v = kyi * gxv - (dg ? kxi * kyi : mk(0.0));
    else v = kyi * gyv - C[mo] + (dg ? kxi * kxi : mk(0.0));
    Mb[rc] = to_t<T>(v);
  }
}

// CTAs per problem of the per-problem element-wise kernels: ~2048 elements each, at most 64.
inline unsigned per_problem_blocks(int64_t elems) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((elems + 2047) / 2048, 64));
}

// M = P Q of every problem (k_assemble_pq_t), in launches of at most 65535 problems.
template <typename T>
int launch_assemble_pq(int64_t batch, int nh, const cd* Cm, const cd* Hx, const cd* Hy, const int* midx,
                       const double* gx, const double* gy, const double* kp, const double* k0, cplx<T>* M,
                       cudaStream_t s) {
  const size_t smem = sizeof(cd) * 2 * (size_t)nh;
  if (smem > 48 * 1024) return KHP_ERR_TOO_LARGE;
  for (int64_t off = 0; off < batch; off += 65535) {
    const unsigned nb = (unsigned)std::min<int64_t>(batch - off, 65535);
    k_assemble_pq_t<T><<<dim3(per_problem_blocks(4 * (int64_t)nh * nh), nb), 256, smem, s>>>(off, nh, Cm, Hx, Hy,
                                                                                         midx, gx, gy, kp, k0, M);
    count_launches(1);
  }
  return cuda_status();
}

template <typename T>
__global__ void k_sqrt_lam_t(int64_t count, cplx<T>* lam) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < count; e += (int64_t)gridDim.x * blockDim.x)
    lam[e] = to_t<T>(csqrt(to_d(lam[e])));
}

// V = Q W / lam (alternative.py:167-176), CWt = C W_top, CWb = C W_bottom ([nh][n] each, batch
// stride cws).  One grid row per problem (b = boff + blockIdx.y) with the problem's wave vectors and
// the reciprocals of its lam tabulated in shared memory (dynamic, 4 nh complex); launched by
// launch_modes_v.
template <typename T>
__global__ void k_modes_v_t(int64_t boff, int nh, const double* gx, const double* gy, const double* kp,
                            const double* k0, const cplx<T>* __restrict__ W, const cplx<T>* __restrict__ CWt,
                            const cplx<T>* __restrict__ CWb, int64_t cws, const cplx<T>* __restrict__ lam, cplx<T>* V,
                            int* status) {
  extern __shared__ cd kt_v[];
  const int n = 2 * nh, nn = n * n;
  cd* kxs = kt_v;
  cd* kys = kxs + nh;
  cd* il = kys + nh;  // 1 / lam[c]
  const int64_t b = boff + blockIdx.y;
  for (int g = threadIdx.x; g < nh; g += blockDim.x) phys::kvec(kp, k0, gx, gy, b, g, kxs[g], kys[g]);
  for (int c = threadIdx.x; c < n; c += blockDim.x) il[c] = cdiv(mk(1.0), to_d(lam[b * n + c]));
  __syncthreads();
  const cplx<T>* Wb = W + b * (int64_t)nn;
  const cplx<T>* Ct = CWt + b * cws;
  const cplx<T>* Cb = CWb + b * cws;
  cplx<T>* Vb = V + b * (int64_t)nn;
  bool bad = false;
  for (int rc = blockIdx.x * blockDim.x + threadIdx.x; rc < nn; rc += gridDim.x * blockDim.x) {
    const int r = rc / n, c = rc - r * n;
    const int i = r < nh ? r : r - nh;
    const cd kx = kxs[i], ky = kys[i];
    const cd wt = to_d(Wb[(int64_t)i * n + c]), wb = to_d(Wb[(int64_t)(nh + i) * n + c]);
    const cd kxy = kx * ky;
    cd q;
    if (r < nh) q = kxy * wt - kx * kx * wb + to_d(Cb[(int64_t)i * n + c]);
    else q = ky * ky * wt - to_d(Ct[(int64_t)i * n + c]) - kxy * wb;
    const cd v = q * il[c];
    Vb[rc] = to_t<T>(v);
    bad |= !cfinite(v);
  }
  if (bad) atomicOr(status + b, KHP_BIT_NONFINITE);
}

template <typename T>
int launch_modes_v(int64_t batch, int nh, const double* gx, const double* gy, const double* kp, const double* k0,
                   const cplx<T>* W, const cplx<T>* CWt, const cplx<T>* CWb, int64_t cws, const cplx<T>* lam,
                   cplx<T>* V, int* status, cudaStream_t s) {
  const size_t smem = sizeof(cd) * 4 * (size_t)nh;
  if (smem > 48 * 1024) return KHP_ERR_TOO_LARGE;
  for (int64_t off = 0; off < batch; off += 65535) {
    const unsigned nb = (unsigned)std::min<int64_t>(batch - off, 65535);
    k_modes_v_t<T><<<dim3(per_problem_blocks(4 * (int64_t)nh * nh), nb), 256, smem, s>>>(off, nh, gx, gy, kp, k0, W,
                                                                                    CWt, CWb, cws, lam, V, status);
    count_launches(1);
  }
  return cuda_status();
}

// Free-space V0 blocks and their inverses per problem and harmonic, [batch][nh] (FP64; computed
// once so that the element-wise products below do no square roots or divisions).
__global__ void k_v0_blocks(int64_t batch, int nh, const double* gx, const double* gy, const double* kp,
                            const double* k0, M2* v0, M2* v0i) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < batch * nh; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / nh;
    const int g = (int)(e % nh);
    cd kx, ky;
    phys::kvec(kp, k0, gx, gy, b, g, kx, ky);
    const M2 v = phys::v0_block(kx, ky);
    v0[e] = v;
    v0i[e] = phys::inv2(v);
  }
}

// out = A V0 (V0: free-space modes, one 2x2 block per harmonic, from k_v0_blocks).
template <typename T>
__global__ void k_v0_right(int64_t batch, int nh, const M2* __restrict__ v0b, const cplx<T>* __restrict__ A,
                           cplx<T>* out) {
  const int n = 2 * nh;
  const int64_t nn = (int64_t)n * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < batch * nn; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / nn;
    const int rc = (int)(e % nn);
    const int r = rc / n, c = rc % n;
    const int g = c % nh, cb = c / nh;
    const M2& v0 = v0b[b * nh + g];
    const cd a0 = to_d(A[b * nn + (int64_t)r * n + g]), a1 = to_d(A[b * nn + (int64_t)r * n + nh + g]);
    out[e] = to_t<T>(a0 * blk(v0, 0, cb) + a1 * blk(v0, 1, cb));
  }
}

// out = V0^-1 A.
template <typename T>
__global__ void k_v0inv_left(int64_t batch, int nh, const M2* __restrict__ v0ib, const cplx<T>* __restrict__ A,
                             cplx<T>* out) {
  const int n = 2 * nh;
  const int64_t nn = (int64_t)n * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < batch * nn; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / nn;
    const int rc = (int)(e % nn);
    const int r = rc / n, c = rc % n;
    const int g = r % nh, rb = r / nh;
    const M2& vi = v0ib[b * nh + g];
    const cd a0 = to_d(A[b * nn + (int64_t)g * n + c]), a1 = to_d(A[b * nn + (int64_t)(nh + g) * n + c]);
    out[e] = to_t<T>(blk(vi, rb, 0) * a0 + blk(vi, rb, 1) * a1);
  }
}

// Homogeneous media: per problem and harmonic the four 2x2 blocks of S (double), [batch][nh][4].
__global__ void k_homog_blocks(int64_t batch, int nh, int kind, cd eps, DepthSel depth, const double* gx, const double* gy,
                               const double* kp, const double* k0, M2* out, int* status) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < batch * nh; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / nh;
    const int g = (int)(e % nh);
    cd kx, ky;
    phys::kvec(kp, k0, gx, gy, b, g, kx, ky);
    M2 s[4], vm;
    cd lm;
    phys::homogeneous_blocks(kind, kx, ky, eps, depth.at(b) * k0[b], s, vm, lm);
    bool fin = true;
    for (int q = 0; q < 4; ++q) {
      out[e * 4 + q] = s[q];
      fin = fin && cfinite(s[q].a) && cfinite(s[q].b) && cfinite(s[q].c) && cfinite(s[q].d);
    }
    if (!fin) atomicOr(status + b, KHP_BIT_NONFINITE);
  }
}

// Gamma = S11 of a homogeneous medium, densely.
template <typename T>
__global__ void k_gamma_from_blocks(int64_t batch, int nh, const M2* __restrict__ S, int q, cplx<T>* G) {
  const int n = 2 * nh;
  const int64_t nn = (int64_t)n * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < batch * nn; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / nn;
    const int rc = (int)(e % nn);
    const int r = rc / n, c = rc % n;
    const int gi = r % nh, gj = c % nh;
    G[e] = gi == gj ? to_t<T>(blk(S[(b * nh + gi) * 4 + q], r / nh, c / nh)) : mk(T(0));
  }
}

// A 2x2 block in the output precision (per-problem tables of the kernels below).
template <typename T>
struct M2t {
  cplx<T> a, b, c, d;
};
template <typename T>
__device__ __forceinline__ M2t<T> to_m2t(const M2& m) {
  return M2t<T>{to_t<T>(m.a), to_t<T>(m.b), to_t<T>(m.c), to_t<T>(m.d)};
}
template <typename T>
__device__ __forceinline__ cplx<T> blkt(const M2t<T>& m, int r, int c) {
  return r == 0 ? (c == 0 ? m.a : m.b) : (c == 0 ? m.c : m.d);
}

// out = I - S22 Gamma (S22 per-harmonic blocks), in T.  One grid row per problem (b = boff +
// blockIdx.y), the problem's S22 blocks tabulated in shared memory; launch_i_minus_sg.
template <typename T>
__global__ void k_i_minus_sg(int64_t boff, int nh, const M2* __restrict__ S, const cplx<T>* __restrict__ G,
                             cplx<T>* out) {
  extern __shared__ unsigned char kt_sg[];
  M2t<T>* s22 = reinterpret_cast<M2t<T>*>(kt_sg);
  const int64_t b = boff + blockIdx.y;
  for (int g = threadIdx.x; g < nh; g += blockDim.x) s22[g] = to_m2t<T>(S[(b * nh + g) * 4 + 3]);
  __syncthreads();
  const int n = 2 * nh, nn = n * n;
  const cplx<T>* Gb = G + b * (int64_t)nn;
  cplx<T>* ob = out + b * (int64_t)nn;
  for (int rc = blockIdx.x * blockDim.x + threadIdx.x; rc < nn; rc += gridDim.x * blockDim.x) {
    const int r = rc / n, c = rc - r * n;
    const int rb = r >= nh ? 1 : 0, g = r - rb * nh;
    const M2t<T> m = s22[g];
    const cplx<T> v = blkt(m, rb, 0) * Gb[(int64_t)g * n + c] + blkt(m, rb, 1) * Gb[(int64_t)(nh + g) * n + c];
    ob[rc] = (r == c ? mk(T(1)) : mk(T(0))) - v;
  }
}

// out = S11 + S12 Z S21 (all S blocks per-harmonic), in T; layout as k_i_minus_sg, the problem's
// S11, S12 and S21 blocks tabulated; launch_sandwich.
template <typename T>
__global__ void k_sandwich(int64_t boff, int nh, const M2* __restrict__ S, const cplx<T>* __restrict__ Z,
                           cplx<T>* out) {
  extern __shared__ unsigned char kt_sw[];
  M2t<T>* s11 = reinterpret_cast<M2t<T>*>(kt_sw);
  M2t<T>* s12 = s11 + nh;
  M2t<T>* s21 = s12 + nh;
  const int64_t b = boff + blockIdx.y;
  for (int g = threadIdx.x; g < nh; g += blockDim.x) {
    const M2* Sg = S + (b * nh + g) * 4;
    s11[g] = to_m2t<T>(Sg[0]);
    s12[g] = to_m2t<T>(Sg[1]);
    s21[g] = to_m2t<T>(Sg[2]);
  }
  __syncthreads();
  const int n = 2 * nh, nn = n * n;
  const cplx<T>* Zb = Z + b * (int64_t)nn;
  cplx<T>* ob = out + b * (int64_t)nn;
  for (int rc = blockIdx.x * blockDim.x + threadIdx.x; rc < nn; rc += gridDim.x * blockDim.x) {
    const int r = rc / n, c = rc - r * n;
    const int ri = r >= nh ? 1 : 0, cj = c >= nh ? 1 : 0;
    const int gi = r - ri * nh, gj = c - cj * nh;
    const M2t<T> sj = s21[gj];
    cplx<T> acc = gi == gj ? blkt(s11[gi], ri, cj) : mk(T(0));
    for (int ra = 0; ra < 2; ++ra) {
      const cplx<T> sv = blkt(s12[gi], ri, ra);
      const int a = ra * nh + gi;
      const cplx<T> z0 = Zb[(int64_t)a * n + gj], z1 = Zb[(int64_t)a * n + nh + gj];
      acc += sv * (z0 * blkt(sj, 0, cj) + z1 * blkt(sj, 1, cj));
    }
    ob[rc] = acc;
  }
}

template <typename T>
int launch_i_minus_sg(int64_t batch, int nh, const M2* S, const cplx<T>* G, cplx<T>* out, cudaStream_t s) {
  const size_t smem = sizeof(M2t<T>) * (size_t)nh;
  if (smem > 48 * 1024) return KHP_ERR_TOO_LARGE;
  for (int64_t off = 0; off < batch; off += 65535) {
    const unsigned nb = (unsigned)std::min<int64_t>(batch - off, 65535);
    k_i_minus_sg<T><<<dim3(per_problem_blocks(4 * (int64_t)nh * nh), nb), 256, smem, s>>>(off, nh, S, G, out);
    count_launches(1);
  }
  return cuda_status();
}

template <typename T>
int launch_sandwich(int64_t batch, int nh, const M2* S, const cplx<T>* Z, cplx<T>* out, cudaStream_t s) {
  const size_t smem = sizeof(M2t<T>) * 3 * (size_t)nh;
  if (smem > 48 * 1024) return KHP_ERR_TOO_LARGE;
  for (int64_t off = 0; off < batch; off += 65535) {
    const unsigned nb = (unsigned)std::min<int64_t>(batch - off, 65535);
    k_sandwich<T><<<dim3(per_problem_blocks(4 * (int64_t)nh * nh), nb), 256, smem, s>>>(off, nh, S, Z, out);
    count_launches(1);
  }
  return cuda_status();
}

// A = F - G (into a), B = F + G (into f).
template <typename T>
__global__ void k_diff_sum(int64_t count, cplx<T>* f, const cplx<T>* __restrict__ g, cplx<T>* a) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < count; e += (int64_t)gridDim.x * blockDim.x) {
    const cplx<T> fv = f[e], gv = g[e];
    a[e] = fv - gv;
    f[e] = fv + gv;
  }
}

// x = exp(-lam k0 d) per problem and mode, [batch][n].
template <typename T>
__global__ void k_xvec(int64_t batch, int n, const cplx<T>* __restrict__ lam, DepthSel depth, const double* k0,
                       cplx<T>* xv) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < batch * n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / n;
    xv[e] = to_t<T>(cexp(-(to_d(lam[e]) * (depth.at(b) * k0[b]))));
  }
}

// rho <- X rho X with X = diag(xv) from k_xvec.
template <typename T>
__global__ void k_xmx_t(int64_t batch, int n, const cplx<T>* __restrict__ xv, cplx<T>* M) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < batch * nn; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / nn;
    const int rc = (int)(e % nn);
    M[e] = xv[b * n + rc / n] * M[e] * xv[b * n + rc % n];
  }
}

// Two-column vectors [batch][n][2].
// u = S21 columns c0 and nh + c0 of a homogeneous medium (its response to the unit sources).
template <typename T>
__global__ void k_src_cols(int64_t batch, int nh, const M2* __restrict__ S, int q, cplx<T>* u) {
  const int n = 2 * nh;
  const int c0 = (nh - 1) / 2;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < batch * n * 2; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / (2 * n);
    const int r = (int)((e / 2) % n), col = (int)(e % 2);
    const int g = r % nh;
    u[e] = g == c0 ? to_t<T>(blk(S[(b * nh + g) * 4 + q], r / nh, col)) : mk(T(0));
  }
}

// out = S_q u (+ S_p columns of the unit sources when add_src >= 0).
template <typename T>
__global__ void k_block_apply(int64_t batch, int nh, const M2* __restrict__ S, int q, const cplx<T>* __restrict__ u,
                              cplx<T>* out, int add_src) {
  const int n = 2 * nh;
  const int c0 = (nh - 1) / 2;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < batch * n * 2; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / (2 * n);
    const int r = (int)((e / 2) % n), col = (int)(e % 2);
    const int g = r % nh, rb = r / nh;
    const M2& s = S[(b * nh + g) * 4 + q];
    const cplx<T>* ub = u + b * n * 2;
    cd v = blk(s, rb, 0) * to_d(ub[g * 2 + col]) + blk(s, rb, 1) * to_d(ub[(nh + g) * 2 + col]);
    if (add_src >= 0 && g == c0) v += blk(S[(b * nh + g) * 4 + add_src], rb, col);
    out[e] = to_t<T>(v);
  }
}

// u <- 4 X u (patterned layer, forward pass).
template <typename T>
__global__ void k_vec_x4(int64_t batch, int n, const cplx<T>* __restrict__ lam, DepthSel depth, const double* k0,
                         cplx<T>* u) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < batch * n * 2; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / (2 * n);
    const int r = (int)((e / 2) % n);
    const cd x = cexp(-(to_d(lam[b * n + r]) * (depth.at(b) * k0[b])));
    u[e] = to_t<T>((4.0 * x) * to_d(u[e]));
  }
}

// R, T from the two source columns of r and t ([batch][n][2]) for npol polarisations
// (te, tm: [batch][npol]; R, T: [batch][npol]), one CTA per problem.
template <typename T>
__global__ void k_flux_cols(int nh, int npol, const cplx<T>* __restrict__ rv, const cplx<T>* __restrict__ tv,
                            const double* gx, const double* gy, const double* kp, const double* k0v, const cd* te_v,
                            const cd* tm_v, cd epsi, cd epse, double* R, double* Tt) {
  __shared__ TeamShared sh;
  TeamCta t;
  const int64_t b = blockIdx.x;
  const int n = 2 * nh;
  const double k0 = k0v[b];
  const cd kpx = mk(kp[4 * b + 0], kp[4 * b + 1]), kpy = mk(kp[4 * b + 2], kp[4 * b + 3]);
  const cd kzi_abs = conj(csqrt(mk(k0 * k0) * epsi - kpx * kpx - kpy * kpy));
  const cd kzi_n = kzi_abs * (1.0 / k0);
  for (int pol = 0; pol < npol; ++pol) {
    cd px, py;
    phys::source_pol(kpx, kpy, kzi_abs, te_v[b * npol + pol], tm_v[b * npol + pol], px, py);
    double rs = 0.0, ts = 0.0;
    for (int g = t.tid(); g < nh; g += t.size()) {
      const cd kxa = mk(kp[4 * b + 0] + gx[g], kp[4 * b + 1]);
      const cd kya = mk(kp[4 * b + 2] + gy[g], kp[4 * b + 3]);
      const cd kx = kxa * (1.0 / k0), ky = kya * (1.0 / k0);
      for (int which = 0; which < 2; ++which) {
        const cplx<T>* v = (which == 0 ? rv : tv) + b * n * 2;
        const cd eps = which == 0 ? epsi : epse;
        const cd kz = conj(csqrt(mk(k0 * k0) * conj(eps) - kxa * kxa - kya * kya)) * (1.0 / k0);
        const cd sx = to_d(v[g * 2 + 0]) * px + to_d(v[g * 2 + 1]) * py;
        const cd sy = to_d(v[(nh + g) * 2 + 0]) * px + to_d(v[(nh + g) * 2 + 1]) * py;
        const cd sz = -cdiv(kx * sx + ky * sy, kz);
        const double tg = kz.re / kzi_n.re * (norm2(sx) + norm2(sy) + norm2(sz));
        if (which == 0) rs += tg;
        else ts += tg;
      }
    }
    rs = team_sum(t, rs, &sh);
    ts = team_sum(t, ts, &sh);
    if (threadIdx.x == 0) {
      R[b * npol + pol] = rs;
      Tt[b * npol + pol] = ts;
    }
  }
}

}  // namespace
}  // namespace khp
