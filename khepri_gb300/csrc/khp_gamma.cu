// Batched reflection / transmission by a backward reflection-matrix recursion (khp_solve_batched).
//
// The reference builds every layer's S-matrix (alternative.build_scatmat, alternative.py:181-195)
// and chains them with four-block Redheffer products (alternative.py:19-30, layer.py:35-60),
// then reads R and T from two blocks of the global S (crystal.py:363-396).  R and T only need
// the global S11 and S21 applied to the incident vector, so this pipeline computes instead:
//
//   backward, from the emergence side:  Gamma = reflection matrix of everything to the right of
//   a free-space gap.  Through a homogeneous medium with (closed-form, per-harmonic) S-matrix:
//       M = I - S22 Gamma,  Gamma <- S11 + S12 (Gamma M^-1) S21;
//   through a patterned layer (modes W, V, lam; X = exp(-lam k0 d)), in its own mode basis:
//       F = W^-1 (I + Gamma), G = V^-1 V0 (Gamma - I), rho = (F + G)(F - G)^-1,
//       rho_L = X rho X, P1 = W (I + rho_L), P2 = V0^-1 V (rho_L - I),
//       Gamma <- (P1 + P2)(P1 - P2)^-1;
//   forward, from the incidence side, the right-going amplitudes of the two source columns:
//       homogeneous: u <- M^-1 S21 u;  patterned: u <- 2 (F - G)^-1 X 2 (P1 - P2)^-1 u,
//   with the LU factors kept from the backward pass; finally r = S11 c + S12 Gamma u at the
//   incidence half-space and t = S21 u at the emergence half-space.
//
// Exactly equivalent to the reference's chain (same continuity conditions), ~2.8x fewer flops
// at 11x11, and only exponentially decaying propagators X appear.  Patterned layers that share a
// pixmap share one eigensolve and the inverses W^-1, V^-1 per problem.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "khepri_gb300.h"
#include "khp_dense.cuh"
#include "khp_launch.h"
#include "khp_physics.cuh"
#include "khp_gamma_kernels.cuh"

namespace khp {
namespace {

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

template <typename T>
struct GammaPlan {
  // per distinct map
  std::vector<cplx<T>*> W, V, lam, Wi, Q0, Vt;
  // modes scratch (reused per map)
  cplx<T> *M, *Z, *CW, *lu;
  int* piv;
  std::vector<int*> midx;  // per distinct map: the map index of every problem
  // per layer
  std::vector<cplx<T>*> lu1, lu2;
  std::vector<int*> piv1, piv2;
  std::vector<M2*> blocks;  // homogeneous layers
  M2 *inc, *trn;
  cplx<T> *G, *F, *Gb, *P;
  cplx<T> *u, *tmp, *rv, *tv;
  int* pivs;
  M2 *v0b, *v0ib;  // free-space blocks per problem and harmonic
};

template <typename T>
GammaPlan<T> plan_gamma(Arena& a, int64_t batch, int nh, int nlayers, const int* kinds, int nmaps_used) {
  const size_t n = 2 * (size_t)nh, nn = n * n;
  GammaPlan<T> p;
  for (int m = 0; m < nmaps_used; ++m) {
    p.W.push_back(a.take<cplx<T>>(batch * nn));
    p.V.push_back(a.take<cplx<T>>(batch * nn));
    p.lam.push_back(a.take<cplx<T>>(batch * n));
    p.Wi.push_back(a.take<cplx<T>>(batch * nn));
    p.Q0.push_back(a.take<cplx<T>>(batch * nn));
    p.Vt.push_back(a.take<cplx<T>>(batch * nn));
    p.midx.push_back(a.take<int>(batch));
  }
  p.M = a.take<cplx<T>>(batch * nn);
  p.Z = a.take<cplx<T>>(batch * nn);
  p.CW = a.take<cplx<T>>(batch * nn);
  p.lu = a.take<cplx<T>>(batch * nn);
  p.piv = a.take<int>(batch * n);
  for (int l = 0; l < nlayers; ++l) {
    if (kinds[l] == 1) {
      p.lu1.push_back(a.take<cplx<T>>(batch * nn));
      p.lu2.push_back(a.take<cplx<T>>(batch * nn));
      p.piv1.push_back(a.take<int>(batch * n));
      p.piv2.push_back(a.take<int>(batch * n));
      p.blocks.push_back(nullptr);
    } else {
      p.lu1.push_back(a.take<cplx<T>>(batch * nn));
      p.lu2.push_back(nullptr);
      p.piv1.push_back(a.take<int>(batch * n));
      p.piv2.push_back(nullptr);
      p.blocks.push_back(a.take<M2>(batch * nh * 4));
    }
  }
  p.inc = a.take<M2>(batch * nh * 4);
  p.trn = a.take<M2>(batch * nh * 4);
  p.G = a.take<cplx<T>>(batch * nn);
  p.F = a.take<cplx<T>>(batch * nn);
  p.Gb = a.take<cplx<T>>(batch * nn);
  p.P = a.take<cplx<T>>(batch * nn);
  p.u = a.take<cplx<T>>(batch * n * 2);
  p.tmp = a.take<cplx<T>>(batch * n * 2);
  p.rv = a.take<cplx<T>>(batch * n * 2);
  p.tv = a.take<cplx<T>>(batch * n * 2);
  p.pivs = a.take<int>(batch * n);
  p.v0b = a.take<M2>(batch * nh);
  p.v0ib = a.take<M2>(batch * nh);
  return p;
}

template <typename T>
int launch_getrs_right(int64_t batch, int n, const cplx<T>* A, int64_t lda, int64_t bsA, const int* piv, cplx<T>* B,
                       int64_t ldb, int64_t bsB, int m, cudaStream_t s) {
  k_getrs_right<T><<<(unsigned)batch, 256, 0, s>>>(n, A, lda, bsA, piv, B, ldb, bsB, m);
  count_launches(1);
  return cuda_status();
}

#define GT_TRY(x)        \
  do {                   \
    const int _s = (x);  \
    if (_s) return _s;   \
  } while (0)
#define GT_EW(kernel, total, ...)                                        \
  do {                                                                   \
    kernel<<<grid_for(total), 256, 0, s>>>(__VA_ARGS__);                 \
    count_launches(1);                                                   \
    GT_TRY(cuda_status());                                               \
  } while (0)

// Modes computed elsewhere (the refined FP64 modes of a mixed-precision solve): slot m of
// problem b is row idx[b] of [slots][src_batch] arrays W, V ([n][n]) and lam ([n]).
struct GivenModes {
  const cd* W;
  const cd* V;
  const cd* lam;
  int64_t src_batch;
  const int* idx;
};

// Wd, Vd, lamd of every problem from slot `slot` of the given modes; an index outside
// [0, src_batch) sets KHP_BIT_BAD_INPUT and leaves zeros (then a singular W is reported too).
__global__ void k_gather_modes(int64_t batch, int n, GivenModes g, int slot, cd* Wd, cd* Vd, cd* lamd, int* status) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < batch * nn;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / nn, r = e - b * nn;
    const int src = g.idx[b];
    const bool ok = src >= 0 && src < g.src_batch;
    const int64_t row = ok ? (int64_t)slot * g.src_batch + src : 0;
    Wd[e] = ok ? g.W[row * nn + r] : mk(0.0);
    Vd[e] = ok ? g.V[row * nn + r] : mk(0.0);
    if (r < n) lamd[b * n + r] = ok ? g.lam[row * n + r] : mk(0.0);
    if (!ok && r == 0) atomicOr(status + b, KHP_BIT_BAD_INPUT);
  }
}

template <typename T>
int solve_gamma(int64_t batch, int px, int py, int nlayers, const int* kinds, const int* maps, const double* eps,
                const double* depths, const int* pmap, const double* pdepth, int64_t nmaps, const double* conv,
                const double* hx, const double* hy, const double* gx, const double* gy, cd epsi, cd epse,
                const double* kp, const double* k0, int npol, const double* te, const double* tm, double* R,
                double* Tt, int* status, void* workspace, size_t ws_bytes, cudaStream_t s,
                const GivenModes* given = nullptr) {
  static_assert(sizeof(T) == sizeof(double), "the FP64 recursion reads the caller's FP64 maps directly");
  const int nh = px * py, n = 2 * nh;
  const int64_t nn = (int64_t)n * n, hh = (int64_t)nh * nh, hn = (int64_t)nh * n;
  // distinct maps in use, in order of first appearance
  std::vector<int> used, first;
  std::vector<int> slot(nlayers, -1);
  for (int l = 0; l < nlayers; ++l) {
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
  GammaPlan<T> p = plan_gamma<T>(a, batch, nh, nlayers, kinds, (int)used.size());
  if (!a.ok || !workspace) return KHP_ERR_WORKSPACE;
  const cplx<T> one = mk(T(1)), zero = mk(T(0)), mone = mk(T(-1));

  GT_EW(k_v0_blocks, batch * nh, batch, nh, gx, gy, kp, k0, p.v0b, p.v0ib);
  // ---- modes of every distinct pixmap, and W^-1, V^-1 V0, V0^-1 V ----
  for (size_t m = 0; m < used.size(); ++m) {
    const cd* Cm = reinterpret_cast<const cd*>(conv);
    GT_EW(k_select_maps, batch, batch, pmap ? pmap + (int64_t)first[m] * batch : nullptr, used[m], nmaps, p.midx[m],
          status);
    if (given) {
      GT_EW(k_gather_modes, batch * nn, batch, n, *given, (int)m, p.W[m], p.V[m], p.lam[m], status);
    } else {
      GT_TRY(launch_assemble_pq<T>(batch, nh, Cm, reinterpret_cast<const cd*>(hx), reinterpret_cast<const cd*>(hy),
                                   p.midx[m], gx, gy, kp, k0, p.M, s));
      GT_TRY(launch_geev<T>(batch, n, p.M, n, nn, p.Z, p.W[m], n, nn, p.lam[m], n, status, s));
      GT_EW(k_sqrt_lam_t<T>, batch * n, batch * n, p.lam[m]);
      cplx<T>* CWt = p.CW;
      cplx<T>* CWb = p.CW + batch * hn;
      GT_TRY(launch_gemm<T>(batch, nh, n, nh, one, Cm, nh, hh, p.W[m], n, nn, zero, CWt, n, hn, s, p.midx[m]));
      GT_TRY(launch_gemm<T>(batch, nh, n, nh, one, Cm, nh, hh, p.W[m] + hn, n, nn, zero, CWb, n, hn, s,
                            p.midx[m]));
      GT_TRY(launch_modes_v<T>(batch, nh, gx, gy, kp, k0, p.W[m], CWt, CWb, hn, p.lam[m], p.V[m], status, s));
    }
    GT_TRY(launch_copy<T>(batch, n, n, p.W[m], n, nn, p.lu, n, nn, s));
    GT_TRY(launch_inverse<T>(batch, n, p.lu, n, nn, p.Wi[m], n, nn, p.piv, status, s));
    GT_TRY(launch_copy<T>(batch, n, n, p.V[m], n, nn, p.lu, n, nn, s));
    GT_TRY(launch_inverse<T>(batch, n, p.lu, n, nn, p.Z, n, nn, p.piv, status, s));  // Z = V^-1
    GT_EW(k_v0_right<T>, batch * nn, batch, nh, p.v0b, p.Z, p.Q0[m]);
    GT_EW(k_v0inv_left<T>, batch * nn, batch, nh, p.v0ib, p.V[m], p.Vt[m]);
  }
  // ---- homogeneous media blocks ----
  GT_EW(k_homog_blocks, batch * nh, batch, nh, 1, epsi, DepthSel{nullptr, 0.0}, gx, gy, kp, k0, p.inc, status);
  GT_EW(k_homog_blocks, batch * nh, batch, nh, 2, epse, DepthSel{nullptr, 0.0}, gx, gy, kp, k0, p.trn, status);
  for (int l = 0; l < nlayers; ++l)
    if (kinds[l] != 1)
      GT_EW(k_homog_blocks, batch * nh, batch, nh, 0, mk(eps[2 * l], eps[2 * l + 1]), depth_of(l), gx, gy, kp, k0,
            p.blocks[l], status);
  // ---- backward pass ----
  GT_EW(k_gamma_from_blocks<T>, batch * nn, batch, nh, p.trn, 0, p.G);
  for (int l = nlayers - 1; l >= 0; --l) {
    if (kinds[l] != 1) {
      GT_TRY(launch_i_minus_sg<T>(batch, nh, p.blocks[l], p.G, p.lu1[l], s));
      GT_TRY(launch_getrf<T>(batch, n, p.lu1[l], n, nn, p.piv1[l], status, s));
      GT_TRY(launch_getrs_right<T>(batch, n, p.lu1[l], n, nn, p.piv1[l], p.G, n, nn, n, s));  // G <- G M^-1
      GT_TRY(launch_sandwich<T>(batch, nh, p.blocks[l], p.G, p.F, s));
      std::swap(p.G, p.F);
    } else {
      const int m = slot[l];
      // F = Wi + Wi G ; Gb = Q0 G - Q0
      GT_TRY(launch_copy<T>(batch, n, n, p.Wi[m], n, nn, p.F, n, nn, s));
      GT_TRY(launch_gemm<T>(batch, n, n, n, one, p.Wi[m], n, nn, p.G, n, nn, one, p.F, n, nn, s));
      GT_TRY(launch_copy<T>(batch, n, n, p.Q0[m], n, nn, p.Gb, n, nn, s));
      GT_TRY(launch_gemm<T>(batch, n, n, n, one, p.Q0[m], n, nn, p.G, n, nn, mone, p.Gb, n, nn, s));
      GT_EW(k_diff_sum<T>, batch * nn, batch * nn, p.F, p.Gb, p.lu1[l]);  // lu1 = F - G, F <- F + G
      GT_TRY(launch_getrf<T>(batch, n, p.lu1[l], n, nn, p.piv1[l], status, s));
      GT_TRY(launch_getrs_right<T>(batch, n, p.lu1[l], n, nn, p.piv1[l], p.F, n, nn, n, s));  // rho
      GT_EW(k_xvec<T>, batch * n, batch, n, p.lam[m], depth_of(l), k0, p.u);                      // scratch
      GT_EW(k_xmx_t<T>, batch * nn, batch, n, p.u, p.F);                                           // rho_L
      GT_TRY(launch_copy<T>(batch, n, n, p.W[m], n, nn, p.Gb, n, nn, s));
      GT_TRY(launch_gemm<T>(batch, n, n, n, one, p.W[m], n, nn, p.F, n, nn, one, p.Gb, n, nn, s));    // P1
      GT_TRY(launch_copy<T>(batch, n, n, p.Vt[m], n, nn, p.P, n, nn, s));
      GT_TRY(launch_gemm<T>(batch, n, n, n, one, p.Vt[m], n, nn, p.F, n, nn, mone, p.P, n, nn, s));   // P2
      GT_EW(k_diff_sum<T>, batch * nn, batch * nn, p.Gb, p.P, p.lu2[l]);  // lu2 = P1 - P2, Gb <- P1 + P2
      GT_TRY(launch_getrf<T>(batch, n, p.lu2[l], n, nn, p.piv2[l], status, s));
      GT_TRY(launch_getrs_right<T>(batch, n, p.lu2[l], n, nn, p.piv2[l], p.Gb, n, nn, n, s));  // new Gamma
      std::swap(p.G, p.Gb);
    }
  }
  // ---- incidence half-space: M0 = I - S22 G, u = M0^-1 S21 c, r = S11 c + S12 G u ----
  GT_TRY(launch_i_minus_sg<T>(batch, nh, p.inc, p.G, p.lu, s));
  GT_TRY(launch_getrf<T>(batch, n, p.lu, n, nn, p.pivs, status, s));
  GT_EW(k_src_cols<T>, batch * n * 2, batch, nh, p.inc, 2, p.u);
  GT_TRY(launch_getrs<T>(batch, n, p.lu, n, nn, p.pivs, p.u, 2, 2 * n, 2, s));
  GT_TRY(launch_gemm<T>(batch, n, 2, n, one, p.G, n, nn, p.u, 2, 2 * n, zero, p.tmp, 2, 2 * n, s));
  GT_EW(k_block_apply<T>, batch * n * 2, batch, nh, p.inc, 1, p.tmp, p.rv, 0);
  // ---- forward pass ----
  for (int l = 0; l < nlayers; ++l) {
    if (kinds[l] != 1) {
      GT_EW(k_block_apply<T>, batch * n * 2, batch, nh, p.blocks[l], 2, p.u, p.tmp, -1);
      GT_TRY(launch_getrs<T>(batch, n, p.lu1[l], n, nn, p.piv1[l], p.tmp, 2, 2 * n, 2, s));
      std::swap(p.u, p.tmp);
    } else {
      const int m = slot[l];
      GT_TRY(launch_getrs<T>(batch, n, p.lu2[l], n, nn, p.piv2[l], p.u, 2, 2 * n, 2, s));
      GT_EW(k_vec_x4<T>, batch * n * 2, batch, n, p.lam[m], depth_of(l), k0, p.u);
      GT_TRY(launch_getrs<T>(batch, n, p.lu1[l], n, nn, p.piv1[l], p.u, 2, 2 * n, 2, s));
    }
  }
  GT_EW(k_block_apply<T>, batch * n * 2, batch, nh, p.trn, 2, p.u, p.tv, -1);
  k_flux_cols<T><<<(unsigned)batch, 128, 0, s>>>(nh, npol, p.rv, p.tv, gx, gy, kp, k0,
                                                  reinterpret_cast<const cd*>(te), reinterpret_cast<const cd*>(tm),
                                                  epsi, epse, R, Tt);
  count_launches(1);
  return cuda_status();
}

}  // namespace
}  // namespace khp

using namespace khp;

extern "C" {

size_t khp_solve_batched_workspace(int64_t batch, int32_t nh, int32_t nlayers, const int32_t* layer_kind,
                                   const int32_t* layer_map) {
  if (batch < 0 || nh < 1 || nlayers < 0 || (nlayers > 0 && (!layer_kind || !layer_map))) return 0;
  int used = 0;
  std::vector<int> seen;
  for (int l = 0; l < nlayers; ++l) {
    if (layer_kind[l] != 1) continue;
    if (std::find(seen.begin(), seen.end(), layer_map[l]) == seen.end()) seen.push_back(layer_map[l]);
  }
  used = (int)seen.size();
  Arena a{nullptr, 0};
  plan_gamma<double>(a, batch, nh, nlayers, layer_kind, used);
  return a.off;
}

int khp_solve_batched(int64_t batch, int32_t px, int32_t py, int32_t nlayers, const int32_t* layer_kind,
                      const int32_t* layer_map, const double* layer_eps, const double* layer_depth,
                      const int32_t* problem_map, const double* problem_depth, int64_t nmaps,
                      const double* conv, const double* hx, const double* hy, const double* gx, const double* gy,
                      double epsi_re, double epsi_im, double epse_re, double epse_im, const double* kp,
                      const double* k0, int32_t npol, const double* te, const double* tm, double* R, double* T,
                      int32_t* status, void* workspace, size_t ws_bytes, void* stream) {
  if (batch < 0 || px < 1 || py < 1 || nlayers < 0 || npol < 1 || !gx || !gy || !kp || !k0 || !te || !tm || !R || !T ||
      !status)
    return KHP_ERR_INVALID_ARG;
  if (nlayers > 0 && (!layer_kind || !layer_map || !layer_eps || !layer_depth)) return KHP_ERR_INVALID_ARG;
  for (int l = 0; l < nlayers; ++l) {
    if (layer_kind[l] != 0 && layer_kind[l] != 1) return KHP_ERR_INVALID_ARG;
    if (layer_kind[l] == 1 && (layer_map[l] < 0 || layer_map[l] >= nmaps || !conv || !hx || !hy))
      return KHP_ERR_INVALID_ARG;
  }
  if (batch == 0) return KHP_OK;
  return solve_gamma<double>(batch, px, py, nlayers, layer_kind, layer_map, layer_eps, layer_depth, problem_map,
                             problem_depth, nmaps, conv, hx, hy, gx, gy, mk(epsi_re, epsi_im), mk(epse_re, epse_im),
                             kp, k0, npol, te, tm, R, T, status, workspace, ws_bytes,
                             reinterpret_cast<cudaStream_t>(stream));
}

int khp_solve_batched_mixed_repair(int64_t batch, int32_t px, int32_t py, int32_t nlayers, const int32_t* layer_kind,
                                   const int32_t* layer_map, const double* layer_eps, const double* layer_depth,
                                   const int32_t* problem_map, const double* problem_depth, int64_t nmaps,
                                   const double* conv, const double* hx, const double* hy, const double* gx,
                                   const double* gy, double epsi_re, double epsi_im, double epse_re, double epse_im,
                                   const double* kp, const double* k0, int32_t npol, const double* te,
                                   const double* tm, int64_t mixed_batch, const int32_t* mixed_index,
                                   const void* mixed_workspace, size_t mixed_ws_bytes, double* R, double* T,
                                   int32_t* status, void* workspace, size_t ws_bytes, void* stream) {
  if (batch < 0 || px < 1 || py < 1 || nlayers < 0 || npol < 1 || !gx || !gy || !kp || !k0 || !te || !tm || !R || !T ||
      !status || mixed_batch < 0 || (batch > 0 && (!mixed_index || !mixed_workspace)))
    return KHP_ERR_INVALID_ARG;
  if (nlayers > 0 && (!layer_kind || !layer_map || !layer_eps || !layer_depth)) return KHP_ERR_INVALID_ARG;
  for (int l = 0; l < nlayers; ++l) {
    if (layer_kind[l] != 0 && layer_kind[l] != 1) return KHP_ERR_INVALID_ARG;
    if (layer_kind[l] == 1 && (layer_map[l] < 0 || layer_map[l] >= nmaps || !conv || !hx || !hy))
      return KHP_ERR_INVALID_ARG;
  }
  if (batch == 0) return KHP_OK;
  GivenModes g{nullptr, nullptr, nullptr, mixed_batch, mixed_index};
  const int st = mixed_modes_in_workspace(mixed_batch, px * py, nlayers, layer_kind, layer_map, mixed_workspace,
                                          mixed_ws_bytes, &g.W, &g.V, &g.lam);
  if (st) return st;
  return solve_gamma<double>(batch, px, py, nlayers, layer_kind, layer_map, layer_eps, layer_depth, problem_map,
                             problem_depth, nmaps, conv, hx, hy, gx, gy, mk(epsi_re, epsi_im), mk(epse_re, epse_im),
                             kp, k0, npol, te, tm, R, T, status, workspace, ws_bytes,
                             reinterpret_cast<cudaStream_t>(stream), g.W ? &g : nullptr);
}

}  // extern "C"
