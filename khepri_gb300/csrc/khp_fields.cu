// Field reconstruction of the Crystal path (khepri/crystal.py:234-343, khepri/fields.py:18-76,
// khepri/fourier.py:136-142), in three launches:
//   khp_fields_amplitudes : one CTA per layer: incident mode vector c1p, the layer's mode
//                           amplitudes [c+; c-] from the forward/reverse chains, and
//                           a = RI^-1 R0 [c+; c-] (RI = [[W, W], [-V, V]], R0 the gap basis);
//   khp_fields_fourier    : one CTA per depth z: f = RI (L(z) o a), longitudinal components;
//   khp_fields_idft       : sum_g f_g exp(i (kx_g x + ky_g y)) on the requested points.
#include <cuda_runtime.h>

#include <algorithm>

#include "khepri_gb300.h"
#include "khp_dense.cuh"
#include "khp_launch.h"

namespace khp {
namespace {

using cd = cplx<double>;
constexpr int kThreads = 256;

__device__ __forceinline__ cd kz_branch_f(cd arg) {
  if (arg.re < 0.0) {
    const cd r = csqrt(-arg);
    return mk(r.im, -r.re);
  }
  return csqrt(arg);
}

// Free-space V0 block of harmonic g: Q0 / (i kz0) (alternative.py:84-99).
__device__ __forceinline__ void v0_block(cd kx, cd ky, cd& a, cd& b, cd& c, cd& d) {
  const cd one = mk(1.0);
  const cd kz0 = kz_branch_f(one - kx * kx - ky * ky);
  const cd il0 = cdiv(one, mk(-kz0.im, kz0.re));
  const cd kxy = kx * ky;
  a = il0 * kxy;
  b = il0 * (one - kx * kx);
  c = il0 * (ky * ky - one);
  d = il0 * (-kxy);
}

__device__ __forceinline__ void kvec1(const double* kp, double k0, const double* gx, const double* gy, int g, cd& kx,
                                      cd& ky) {
  kx = mk((kp[0] + gx[g]) / k0, kp[1] / k0);
  ky = mk((kp[2] + gy[g]) / k0, kp[3] / k0);
}

// Per-layer scratch: F (n x n), Wc, Vc (n x n copies), vectors.
struct AmpWs {
  cd* F;
  cd* Wc;
  cd* Vc;
  cd* vec;  // 6 n
  int* piv;
};

__global__ void __launch_bounds__(kThreads)
    k_fields_amplitudes(int nh, const long long* sl_ptrs, const long long* sr_ptrs, const long long* w_ptrs,
                        const long long* v_ptrs, const cd* __restrict__ vref, const cd* __restrict__ inc,
                        const double* gx, const double* gy, const double* kp, const double* k0p, cd* F_all,
                        cd* Wc_all, cd* Vc_all, cd* vec_all, int* piv_all, cd* amps, int* status) {
  __shared__ TeamShared sh;
  TeamCta t;
  const int l = blockIdx.x;
  const int n = 2 * nh;
  const int64_t nn = (int64_t)n * n;
  const cd* Sl = reinterpret_cast<const cd*>(sl_ptrs[l]);
  const cd* Sr = reinterpret_cast<const cd*>(sr_ptrs[l]);
  const cd* W = reinterpret_cast<const cd*>(w_ptrs[l]);
  const cd* V = reinterpret_cast<const cd*>(v_ptrs[l]);
  cd* F = F_all + l * nn;
  cd* Wc = Wc_all + l * nn;
  cd* Vc = Vc_all + l * nn;
  cd* c1p = vec_all + (int64_t)l * 6 * n;
  cd* cp = c1p + n;
  cd* cm = cp + n;
  cd* bt = cm + n;
  cd* bb = bt + n;
  cd* tmp = bb + n;
  int* piv = piv_all + (int64_t)l * n;
  const double k0 = k0p[0];
  int st = 0;
  // c1p = first half of solve([[I, I], [-Vref, Vref]], [e; h]) = (e - Vref^-1 h) / 2
  for (int e = t.tid(); e < nn; e += t.size()) Vc[e] = vref[e];
  for (int i = t.tid(); i < n; i += t.size()) tmp[i] = inc[n + i];
  t.sync();
  st |= team_getrf(t, Vc, n, n, piv, &sh);
  team_getrs(t, Vc, n, n, piv, tmp, 1, 1);
  for (int i = t.tid(); i < n; i += t.size()) c1p[i] = 0.5 * (inc[i] - tmp[i]);
  t.sync();
  // F = I - Sl22 Sr11 ; c+ = F^-1 Sl21 c1p ; c- = Sr11 c+   (fields.py:18-27)
  const cd* Sl21 = Sl + 2 * nn;
  const cd* Sl22 = Sl + 3 * nn;
  const cd* Sr11 = Sr;
  team_gemm(t, n, n, n, mk(-1.0), Sl22, n, Sr11, n, mk(0.0), F, n);
  for (int i = t.tid(); i < n; i += t.size()) F[(int64_t)i * n + i] += mk(1.0);
  for (int i = t.tid(); i < n; i += t.size()) {
    cd acc = mk(0.0);
    for (int j = 0; j < n; ++j) fma_acc(acc, Sl21[(int64_t)i * n + j], c1p[j]);
    cp[i] = acc;
  }
  t.sync();
  st |= team_getrf(t, F, n, n, piv, &sh);
  team_getrs(t, F, n, n, piv, cp, 1, 1);
  for (int i = t.tid(); i < n; i += t.size()) {
    cd acc = mk(0.0);
    for (int j = 0; j < n; ++j) fma_acc(acc, Sr11[(int64_t)i * n + j], cp[j]);
    cm[i] = acc;
  }
  t.sync();
  // R0 [c+; c-] = [c+ + c-; V0 (c- - c+)]
  for (int g = t.tid(); g < nh; g += t.size()) {
    cd kx, ky, a, b, c, d;
    kvec1(kp, k0, gx, gy, g, kx, ky);
    v0_block(kx, ky, a, b, c, d);
    const cd d0 = cm[g] - cp[g], d1 = cm[nh + g] - cp[nh + g];
    bt[g] = cp[g] + cm[g];
    bt[nh + g] = cp[nh + g] + cm[nh + g];
    bb[g] = a * d0 + b * d1;
    bb[nh + g] = c * d0 + d * d1;
  }
  for (int e = t.tid(); e < nn; e += t.size()) {
    Wc[e] = W[e];
    Vc[e] = V[e];
  }
  t.sync();
  // RI^-1 [bt; bb]: s = W^-1 bt, d = V^-1 bb, a+ = (s - d)/2, a- = (s + d)/2
  st |= team_getrf(t, Wc, n, n, piv, &sh);
  team_getrs(t, Wc, n, n, piv, bt, 1, 1);
  st |= team_getrf(t, Vc, n, n, piv, &sh);
  team_getrs(t, Vc, n, n, piv, bb, 1, 1);
  cd* a = amps + (int64_t)l * 2 * n;
  for (int i = t.tid(); i < n; i += t.size()) {
    a[i] = 0.5 * (bt[i] - bb[i]);
    a[n + i] = 0.5 * (bt[i] + bb[i]);
    if (!cfinite(a[i]) || !cfinite(a[n + i])) st |= KHP_BIT_NONFINITE;
  }
  if (st) atomicOr(status, st);
}

// One CTA per depth: f = RI (L o a), L = [exp(lam zbar), exp(-lam zbar)] clamped at 1e14
// (fields.py:53-62), then sz, uz (fields.py:68-76).  ff[z] = [sx, sy, sz, ux, uy, uz] (nh each).
__global__ void __launch_bounds__(kThreads)
    k_fields_fourier(int nh, const int* __restrict__ slot_of_z, const double* __restrict__ zbar,
                     const long long* w_ptrs, const long long* v_ptrs, const long long* lam_ptrs,
                     const long long* ic_ptrs, const cd* __restrict__ ic_scalar, const cd* __restrict__ amps,
                     const double* gx, const double* gy, const double* kp, const double* k0p, cd* ff) {
  extern __shared__ unsigned char dyn[];
  cd* u = reinterpret_cast<cd*>(dyn);  // 2n: u+ + u-, u- - u+
  cd* f = u + 2 * nh * 2;              // 2n: E then H transverse
  const int z = blockIdx.x;
  const int n = 2 * nh;
  const int s = slot_of_z[z];
  const cd* W = reinterpret_cast<const cd*>(w_ptrs[s]);
  const cd* V = reinterpret_cast<const cd*>(v_ptrs[s]);
  const cd* lam = reinterpret_cast<const cd*>(lam_ptrs[s]);
  const cd* a = amps + (int64_t)s * 2 * n;
  const double zb = zbar[z];
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const cd lz = lam[i] * zb;
    cd p = cexp(lz), m = cexp(-lz);
    const double ap = cabs(p), am = cabs(m);
    if (ap > 1e14) p = p * (1e14 / ap);
    if (am > 1e14) m = m * (1e14 / am);
    const cd up = p * a[i], um = m * a[n + i];
    u[i] = up + um;
    u[n + i] = um - up;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 2 * n; i += blockDim.x) {
    const bool top = i < n;
    const int r = top ? i : i - n;
    const cd* M = top ? W : V;
    const cd* x = top ? u : u + n;
    cd acc = mk(0.0);
    for (int j = 0; j < n; ++j) fma_acc(acc, M[(int64_t)r * n + j], x[j]);
    f[i] = acc;
  }
  __syncthreads();
  const double k0 = k0p[0];
  const cd* IC = reinterpret_cast<const cd*>(ic_ptrs[s]);
  const cd ics = ic_scalar[s];
  cd* out = ff + (int64_t)z * 6 * nh;
  const cd mi = mk(0.0, -1.0);
  for (int g = threadIdx.x; g < nh; g += blockDim.x) {
    cd kx, ky;
    kvec1(kp, k0, gx, gy, g, kx, ky);
    const cd sx = f[g], sy = f[nh + g], ux = f[n + g], uy = f[n + nh + g];
    out[g] = sx;
    out[nh + g] = sy;
    out[3 * nh + g] = ux;
    out[4 * nh + g] = uy;
    out[5 * nh + g] = mi * (kx * sy - ky * sx);
    cd q;
    if (IC) {
      q = mk(0.0);
      for (int j = 0; j < nh; ++j) {
        cd kxj, kyj;
        kvec1(kp, k0, gx, gy, j, kxj, kyj);
        fma_acc(q, IC[(int64_t)g * nh + j], kxj * f[n + nh + j] - kyj * f[n + j]);
      }
    } else {
      q = ics * (kx * uy - ky * ux);
    }
    out[2 * nh + g] = mi * q;
  }
}

// out[r][p] = sum_g ff[r][g] exp(i (kx_g x_p + ky_g y_p)), kx_g = kp_x + gx_g (absolute).
// Thread per point, RT rows per thread; phases computed on the fly.
template <int RT>
__global__ void k_fields_idft(int64_t rows, int nh, const cd* __restrict__ ff, const double* gx, const double* gy,
                              const double* kp, int64_t npts, const double* __restrict__ x,
                              const double* __restrict__ y, cd* out) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t r0 = (int64_t)blockIdx.y * RT;
  if (p >= npts) return;
  const double xp = x[p], yp = y[p];
  cd acc[RT];
#pragma unroll
  for (int r = 0; r < RT; ++r) acc[r] = mk(0.0);
  const cd kpx = mk(kp[0], kp[1]), kpy = mk(kp[2], kp[3]);
  for (int g = 0; g < nh; ++g) {
    const cd arg = (kpx + mk(gx[g])) * xp + (kpy + mk(gy[g])) * yp;  // phase = exp(i arg)
    const cd ph = cexp(mk(-arg.im, arg.re));
#pragma unroll
    for (int r = 0; r < RT; ++r)
      if (r0 + r < rows) fma_acc(acc[r], ff[(r0 + r) * nh + g], ph);
  }
#pragma unroll
  for (int r = 0; r < RT; ++r)
    if (r0 + r < rows) out[(r0 + r) * npts + p] = acc[r];
}

}  // namespace
}  // namespace khp

using namespace khp;

extern "C" {

size_t khp_fields_amplitudes_workspace(int64_t nlayers, int32_t nh) {
  const size_t n = 2 * (size_t)nh, nn = n * n;
  auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
  return al(nlayers * nn * sizeof(cd)) * 3 + al(nlayers * 6 * n * sizeof(cd)) + al(nlayers * n * sizeof(int));
}

int khp_fields_amplitudes(int64_t nlayers, int32_t nh, const int64_t* sl_ptrs, const int64_t* sr_ptrs,
                          const int64_t* w_ptrs, const int64_t* v_ptrs, const double* vref, const double* inc,
                          const double* gx, const double* gy, const double* kp, const double* k0, double* amps,
                          int32_t* status, void* workspace, size_t ws_bytes, void* stream) {
  if (nlayers < 0 || nh < 1 || !sl_ptrs || !sr_ptrs || !w_ptrs || !v_ptrs || !vref || !inc || !gx || !gy || !kp ||
      !k0 || !amps || !status)
    return KHP_ERR_INVALID_ARG;
  if (nlayers == 0) return KHP_OK;
  if (!workspace || ws_bytes < khp_fields_amplitudes_workspace(nlayers, nh)) return KHP_ERR_WORKSPACE;
  const size_t n = 2 * (size_t)nh, nn = n * n;
  auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
  char* p = static_cast<char*>(workspace);
  cd* F = reinterpret_cast<cd*>(p);
  p += al(nlayers * nn * sizeof(cd));
  cd* Wc = reinterpret_cast<cd*>(p);
  p += al(nlayers * nn * sizeof(cd));
  cd* Vc = reinterpret_cast<cd*>(p);
  p += al(nlayers * nn * sizeof(cd));
  cd* vec = reinterpret_cast<cd*>(p);
  p += al(nlayers * 6 * n * sizeof(cd));
  int* piv = reinterpret_cast<int*>(p);
  k_fields_amplitudes<<<(unsigned)nlayers, kThreads, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      nh, (const long long*)sl_ptrs, (const long long*)sr_ptrs, (const long long*)w_ptrs, (const long long*)v_ptrs,
      (const cd*)vref, (const cd*)inc, gx, gy, kp, k0, F, Wc, Vc, vec, piv, (cd*)amps, status);
  count_launches(1);
  return cuda_status();
}

int khp_fields_fourier(int64_t nz, int32_t nh, const int32_t* slot_of_z, const double* zbar, const int64_t* w_ptrs,
                       const int64_t* v_ptrs, const int64_t* lam_ptrs, const int64_t* ic_ptrs, const double* ic_scalar,
                       const double* amps, const double* gx, const double* gy, const double* kp, const double* k0,
                       double* ff, void* stream) {
  if (nz < 0 || nh < 1 || !slot_of_z || !zbar || !w_ptrs || !v_ptrs || !lam_ptrs || !ic_ptrs || !ic_scalar || !amps ||
      !gx || !gy || !kp || !k0 || !ff)
    return KHP_ERR_INVALID_ARG;
  if (nz == 0) return KHP_OK;
  const size_t smem = sizeof(cd) * 4 * 2 * (size_t)nh;
  if (smem > 200 * 1024) return KHP_ERR_TOO_LARGE;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute(k_fields_fourier, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return KHP_ERR_CUDA;
  k_fields_fourier<<<(unsigned)nz, kThreads, smem, s>>>(nh, slot_of_z, zbar, (const long long*)w_ptrs,
                                                        (const long long*)v_ptrs, (const long long*)lam_ptrs,
                                                        (const long long*)ic_ptrs, (const cd*)ic_scalar,
                                                        (const cd*)amps, gx, gy, kp, k0, (cd*)ff);
  count_launches(1);
  return cuda_status();
}

int khp_fields_idft(int64_t rows, int32_t nh, const double* ff, const double* gx, const double* gy, const double* kp,
                    int64_t npts, const double* x, const double* y, double* out, void* stream) {
  if (rows < 0 || nh < 1 || npts < 0 || !ff || !gx || !gy || !kp || !x || !y || !out) return KHP_ERR_INVALID_ARG;
  if (rows == 0 || npts == 0) return KHP_OK;
  constexpr int RT = 6;
  const int64_t gy_blocks = (rows + RT - 1) / RT;
  if (gy_blocks > 65535) return KHP_ERR_TOO_LARGE;
  dim3 grid((unsigned)((npts + 127) / 128), (unsigned)gy_blocks);
  k_fields_idft<RT><<<grid, 128, 0, reinterpret_cast<cudaStream_t>(stream)>>>(rows, nh, (const cd*)ff, gx, gy, kp,
                                                                               npts, x, y, (cd*)out);
  count_launches(1);
  return cuda_status();
}

}  // extern "C"
