// RCWA-specific kernels of the Crystal solve and the C-ABI entry points of libkhp.
//
//   convolution matrix  : khepri/tools.py:33-56          -> khp_convmat
//   structure prep      : khepri/layer.py:156-158 (IC)   -> khp_structure_prep
//   patterned modes     : khepri/alternative.py:158-178  -> khp_layer_modes
//   layer S-matrix      : khepri/alternative.py:181-195  -> khp_layer_smatrix
//   homogeneous media   : khepri/alternative.py:32-99, 130-156 -> khp_closed_form_smatrix
//   star product        : khepri/alternative.py:19-30    -> khp_star_product
//   fluxes              : khepri/crystal.py:363-396, alternative.py:101-128, 235-245 -> khp_flux
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "khepri_gb300.h"
#include "khp_dense.cuh"
#include "khp_launch.h"

namespace khp {
namespace {

using cd = cplx<double>;

// ------------------------------------------------------------------------------------------
// Workspace carving: the same plan function runs once to count bytes (base == nullptr) and
// once to hand out pointers.  Every slice starts on a 256-byte boundary.
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

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// ------------------------------------------------------------------------------------------
// Small per-harmonic helpers
// ------------------------------------------------------------------------------------------
struct M2 {
  cd a, b, c, d;  // [[a, b], [c, d]]
};
__device__ __forceinline__ M2 m2(cd a, cd b, cd c, cd d) { return M2{a, b, c, d}; }
__device__ __forceinline__ M2 operator*(const M2& x, const M2& y) {
  return m2(x.a * y.a + x.b * y.c, x.a * y.b + x.b * y.d, x.c * y.a + x.d * y.c, x.c * y.b + x.d * y.d);
}
__device__ __forceinline__ M2 operator+(const M2& x, const M2& y) { return m2(x.a + y.a, x.b + y.b, x.c + y.c, x.d + y.d); }
__device__ __forceinline__ M2 operator-(const M2& x, const M2& y) { return m2(x.a - y.a, x.b - y.b, x.c - y.c, x.d - y.d); }
__device__ __forceinline__ M2 scale(cd s, const M2& x) { return m2(s * x.a, s * x.b, s * x.c, s * x.d); }
__device__ __forceinline__ M2 eye2() { return m2(mk(1.0), mk(0.0), mk(0.0), mk(1.0)); }
__device__ __forceinline__ M2 inv2(const M2& x) {
  const cd det = x.a * x.d - x.b * x.c;
  const cd r = cdiv(mk(1.0), det);
  return m2(r * x.d, -(r * x.b), -(r * x.c), r * x.a);
}
__device__ __forceinline__ bool finite2(const M2& x) {
  return cfinite(x.a) && cfinite(x.b) && cfinite(x.c) && cfinite(x.d);
}

// Normalised in-plane wavevector of harmonic g for problem b: (kp + G) / k0 (expansion.py:43-50).
__device__ __forceinline__ void kvec(const double* kp, const double* k0, const double* gx, const double* gy,
                                     int64_t b, int g, cd& kx, cd& ky) {
  const double k = k0[b];
  kx = mk((kp[4 * b + 0] + gx[g]) / k, kp[4 * b + 1] / k);
  ky = mk((kp[4 * b + 2] + gy[g]) / k, kp[4 * b + 3] / k);
}

// kz with the homogeneous-layer branch: Re(arg) < 0 -> -i sqrt(-arg) (alternative.py:92-96, 145-149).
__device__ __forceinline__ cd kz_branch(cd arg) {
  if (arg.re < 0.0) {
    const cd r = csqrt(-arg);
    return mk(r.im, -r.re);
  }
  return csqrt(arg);
}

// Q of a homogeneous medium of permittivity eps for one harmonic (alternative.py:36-39, 133-135).
__device__ __forceinline__ M2 q_medium(cd kx, cd ky, cd eps) {
  const cd kxy = kx * ky;
  return m2(kxy, eps - kx * kx, ky * ky - eps, -kxy);
}

__device__ __forceinline__ void status_or(int* status, int64_t b, int bits) {
  if (bits) atomicOr(status + b, bits);
}

// ------------------------------------------------------------------------------------------
// Convolution matrix: separable direct DFT of the needed (2px-1) x (2py-1) coefficients,
// then the Toeplitz gather.
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ cd twiddle(int64_t d, int64_t x, int64_t n) {
  int64_t r = (d * x) % n;
  if (r < 0) r += n;
  double s, c;
  sincospi(-2.0 * (double)r / (double)n, &s, &c);
  return mk(c, s);
}

// grid (2px-1, nmaps); dynamic smem ny complex.  F[map][dxi][dyi] = sum eps e^{-2pi i(dx x/nx + dy y/ny)}/(nx ny)
__global__ void k_convmat_dft(int64_t nx, int64_t ny, const cd* __restrict__ eps, int px, int py, cd* F) {
  extern __shared__ unsigned char dyn[];
  cd* g1 = reinterpret_cast<cd*>(dyn);
  const int64_t map = blockIdx.y;
  const int dxi = blockIdx.x;
  const int64_t dx = dxi - (px - 1);
  const cd* e = eps + map * nx * ny;
  for (int64_t y = threadIdx.x; y < ny; y += blockDim.x) {
    cd acc = mk(0.0);
    for (int64_t x = 0; x < nx; ++x) fma_acc(acc, e[x * ny + y], twiddle(dx, x, nx));
    g1[y] = acc;
  }
  __syncthreads();
  const int ndy = 2 * py - 1;
  const double inv = 1.0 / ((double)nx * (double)ny);
  for (int dyi = threadIdx.x; dyi < ndy; dyi += blockDim.x) {
    const int64_t dy = dyi - (py - 1);
    cd acc = mk(0.0);
    for (int64_t y = 0; y < ny; ++y) fma_acc(acc, g1[y], twiddle(dy, y, ny));
    F[(map * (2 * px - 1) + dxi) * ndy + dyi] = acc * inv;
  }
}

__global__ void k_convmat_gather(int64_t nmaps, int px, int py, const cd* __restrict__ F, cd* C) {
  const int nh = px * py, ndx = 2 * px - 1, ndy = 2 * py - 1;
  const int64_t total = nmaps * (int64_t)nh * nh;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t map = e / ((int64_t)nh * nh);
    const int rc = (int)(e % ((int64_t)nh * nh));
    const int r = rc / nh, c = rc % nh;
    const int pr = r % px, qr = r / px, pc = c % px, qc = c / px;
    C[e] = F[(map * ndx + (pr - pc + px - 1)) * ndy + (qr - qc + py - 1)];
  }
}

// (exp(z) - 1) / z with the nested Taylor series below |z| = 1e-2 (fourier.py:7-20).
__device__ cd fexpz(cd z) {
  if (cabs(z) > 1e-2) return cdiv(cexp(z) - mk(1.0), z);
  const cd one = mk(1.0);
  cd r = one + z * (1.0 / 7.0);
  r = one + z * (1.0 / 6.0) * r;
  r = one + z * (1.0 / 5.0) * r;
  r = one + z * (1.0 / 4.0) * r;
  r = one + z * (1.0 / 3.0) * r;
  return one + z * 0.5 * r;
}

// Fourier coefficients of analytical layers (layer.py:161-168, fourier.py:23-58, 145-159) in the
// layout of k_convmat_dft: F[map][dxi][dyi] for |dx| < px, |dy| < py.  The reference evaluates the
// island transforms on the expanded grid epw = (3 px, 3 py) (1 for a single harmonic), lays the
// flat result (m fastest) out as an epw[0] x epw[1] array and reads entry (g0x + dx, g0y + dy);
// the same flat-index arithmetic is used here.  islands: [nisl][8] = map, type (0 disc, 1
// rectangle), eps re, eps im, params[4]; eps_host: complex [nmaps].
__global__ void k_convmat_islands(int64_t nmaps, int px, int py, int nisl, const double* __restrict__ islands,
                                  const cd* __restrict__ eps_host, double b1x, double b1y, double b2x, double b2y,
                                  double sigma, cd* F) {
  const int ndx = 2 * px - 1, ndy = 2 * py - 1;
  const int ex = px > 1 ? 3 * px : 1, ey = py > 1 ? 3 * py : 1;
  const int64_t total = nmaps * (int64_t)ndx * ndy;
  const double pi = 3.14159265358979323846;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t map = e / ((int64_t)ndx * ndy);
    const int k = (int)(e % ((int64_t)ndx * ndy));
    const int dx = k / ndy - (px - 1), dy = k % ndy - (py - 1);
    const int a = ex / 2 + dx, b = ey / 2 + dy;
    const int flat = a * ey + b;
    const int i = flat % ex, j = flat / ex;
    const double m = i - (ex - 1) / 2, nn = j - (ey - 1) / 2;
    const double gx = m * b1x + nn * b2x, gy = m * b1y + nn * b2y;
    const cd host = eps_host[map];
    cd acc = flat == (ex * ey - 1) / 2 ? host : mk(0.0);
    for (int s = 0; s < nisl; ++s) {
      const double* isl = islands + 8 * s;
      if ((int64_t)isl[0] != map) continue;
      const cd coef = mk(isl[2], isl[3]) - host;
      cd tr;
      if (isl[1] == 0.0) {  // disc (center0, center1, radius)
        const double r = isl[6];
        const double norm = sqrt(gx * gx + gy * gy) * r;
        if (fabs(gx) <= 1e-8 && fabs(gy) <= 1e-8) {
          tr = mk(pi * r * r / sigma);
        } else {
          const double ph = -(isl[4] * gx + isl[5] * gy);
          tr = mk(cos(ph), sin(ph)) * (pi * r * r / sigma * 2.0 * j1(norm) / norm);
        }
      } else {  // rectangle (ll0, ll1, ur0, ur1)
        const double w = isl[6] - isl[4], h = isl[7] - isl[5];
        const double ph = -(isl[4] * gx + isl[5] * gy);
        tr = fexpz(mk(0.0, -gx * w)) * fexpz(mk(0.0, -gy * h)) * mk(cos(ph), sin(ph)) * (w * h / sigma);
      }
      acc += coef * tr;
    }
    F[e] = acc;
  }
}

// Adjoint of k_convmat_gather: dF[map][dx][dy] = sum of dC over the (r, c) with
// p_r - p_c = dx, q_r - q_c = dy (fixed order).
__global__ void k_convmat_bwd_gather(int64_t nmaps, int px, int py, const cd* __restrict__ dC, cd* dF) {
  const int nh = px * py, ndx = 2 * px - 1, ndy = 2 * py - 1;
  const int64_t total = nmaps * (int64_t)ndx * ndy;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t map = e / ((int64_t)ndx * ndy);
    const int k = (int)(e % ((int64_t)ndx * ndy));
    const int dx = k / ndy - (px - 1), dy = k % ndy - (py - 1);
    cd acc = mk(0.0);
    for (int qc = 0; qc < py; ++qc) {
      const int qr = qc + dy;
      if (qr < 0 || qr >= py) continue;
      for (int pc = 0; pc < px; ++pc) {
        const int pr = pc + dx;
        if (pr < 0 || pr >= px) continue;
        acc += dC[map * (int64_t)nh * nh + (int64_t)(qr * px + pr) * nh + (qc * px + pc)];
      }
    }
    dF[e] = acc;
  }
}

// Adjoint of k_convmat_dft, first stage: h[map][dxi][y] = sum_dy dF[map][dxi][dy] e^{-2 pi i dy y / ny}.
__global__ void k_convmat_bwd_dft_y(int64_t nmaps, int px, int py, int64_t ny, const cd* __restrict__ dF, cd* h) {
  const int ndx = 2 * px - 1, ndy = 2 * py - 1;
  const int64_t total = nmaps * (int64_t)ndx * ny;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t y = e % ny, md = e / ny;  // md = map * ndx + dxi
    cd acc = mk(0.0);
    for (int dyi = 0; dyi < ndy; ++dyi) fma_acc(acc, dF[md * ndy + dyi], twiddle(dyi - (py - 1), y, ny));
    h[e] = acc;
  }
}

// Second stage: deps[map][x][y] = sum_dx h[map][dxi][y] e^{-2 pi i dx x / nx} / (nx ny).
__global__ void k_convmat_bwd_dft_x(int64_t nmaps, int px, int64_t nx, int64_t ny, const cd* __restrict__ h,
                                    cd* deps) {
  const int ndx = 2 * px - 1;
  const int64_t total = nmaps * nx * ny;
  const double inv = 1.0 / ((double)nx * (double)ny);
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t map = e / (nx * ny);
    const int64_t xy = e % (nx * ny);
    const int64_t x = xy / ny, y = xy % ny;
    cd acc = mk(0.0);
    for (int dxi = 0; dxi < ndx; ++dxi) fma_acc(acc, h[(map * ndx + dxi) * ny + y], twiddle(dxi - (px - 1), x, nx));
    deps[e] = acc * inv;
  }
}

// tmp = diag(g) C  (row scaling), batch of maps
__global__ void k_row_scale_real(int64_t nmaps, int nh, const double* __restrict__ g, const cd* __restrict__ C, cd* out) {
  const int64_t total = nmaps * (int64_t)nh * nh;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)((e / nh) % nh);
    out[e] = C[e] * g[i];
  }
}

// ------------------------------------------------------------------------------------------
// Homogeneous media: closed-form per-harmonic S-matrices (S must be zero-filled beforehand).
// ------------------------------------------------------------------------------------------
__global__ void k_closed_form(int64_t batch, int nh, int kind, const cd* __restrict__ eps, const double* depth,
                              const double* gx, const double* gy, const double* kp, const double* k0, cd* S, cd* W,
                              cd* V, cd* lam, int* status) {
  const int n = 2 * nh;
  const int64_t nn = (int64_t)n * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < batch * nh; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / nh;
    const int g = (int)(e % nh);
    cd kx, ky;
    kvec(kp, k0, gx, gy, b, g, kx, ky);
    const cd one = mk(1.0);
    const cd kz0 = kz_branch(one - kx * kx - ky * ky);
    const cd lam0 = mk(-kz0.im, kz0.re);  // i kz0
    const cd il0 = cdiv(one, lam0);
    const M2 v0 = scale(il0, q_medium(kx, ky, one));
    const cd ep = eps[b];
    M2 s11, s12, s21, s22, vm;
    cd lm;
    if (kind == 0) {
      const cd kz = kz_branch(ep - kx * kx - ky * ky);
      lm = mk(-kz.im, kz.re);
      vm = scale(cdiv(one, lm), q_medium(kx, ky, ep));
      const M2 t2 = inv2(vm) * v0;
      const M2 A = eye2() + t2, B = eye2() - t2;
      const cd x = cexp(-(lm * (depth[b] * k0[b])));
      const cd x2 = x * x;
      const M2 bab = B * inv2(A) * B;
      const M2 tinv = inv2(A - scale(x2, bab));
      s11 = scale(x2 - one, tinv * B);
      s12 = scale(x, tinv * (A - bab));
      s21 = s12;
      s22 = s11;
    } else {
      const cd kz = conj(csqrt(ep - kx * kx - ky * ky));
      lm = mk(-kz.im, kz.re);
      vm = scale(cdiv(one, lm), q_medium(kx, ky, ep));
      const M2 t2 = inv2(v0) * vm;
      const M2 A = eye2() + t2, B = eye2() - t2;
      const M2 ai = inv2(A);
      const M2 aib = ai * B;
      const M2 half = scale(mk(0.5), A - B * aib);
      if (kind == 1) {
        s11 = scale(mk(-1.0), aib);
        s12 = scale(mk(2.0), ai);
        s21 = half;
        s22 = B * ai;
      } else {
        s11 = B * ai;
        s12 = half;
        s21 = scale(mk(2.0), ai);
        s22 = scale(mk(-1.0), aib);
      }
    }
    cd* Sb = S + b * 4 * nn;
    const int r0 = g, r1 = nh + g;
    const M2* blk[4] = {&s11, &s12, &s21, &s22};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      cd* P = Sb + q * nn;
      P[(int64_t)r0 * n + r0] = blk[q]->a;
      P[(int64_t)r0 * n + r1] = blk[q]->b;
      P[(int64_t)r1 * n + r0] = blk[q]->c;
      P[(int64_t)r1 * n + r1] = blk[q]->d;
    }
    if (W) {
      W[b * nn + (int64_t)r0 * n + r0] = one;
      W[b * nn + (int64_t)r1 * n + r1] = one;
    }
    if (V) {
      cd* P = V + b * nn;
      P[(int64_t)r0 * n + r0] = vm.a;
      P[(int64_t)r0 * n + r1] = vm.b;
      P[(int64_t)r1 * n + r0] = vm.c;
      P[(int64_t)r1 * n + r1] = vm.d;
    }
    if (lam) {
      lam[b * n + r0] = lm;
      lam[b * n + r1] = lm;
    }
    const bool fin = finite2(s11) && finite2(s12) && finite2(s21) && finite2(s22);
    if (!fin) status_or(status, b, KHP_BIT_NONFINITE);
  }
}

// ------------------------------------------------------------------------------------------
// Patterned layers
// ------------------------------------------------------------------------------------------
// M = P Q assembled in O(n^2) from C, Hx = C^-1 diag(gx) C, Hy = C^-1 diag(gy) C:
//   M = [[Ky^2 - C + Kx Gx, Kx Gy - Kx Ky], [Ky Gx - Kx Ky, Kx^2 - C + Ky Gy]],
//   Gx = C^-1 Kx C = (kpx/k0) I + Hx/k0,  Gy likewise  (algebraically equal to the reference's
//   P Q product, alternative.py:162-172, because diagonal matrices commute).
__global__ void k_assemble_pq(int64_t batch, int nh, const int* __restrict__ map_index, const cd* __restrict__ C,
                              const cd* __restrict__ Hx, const cd* __restrict__ Hy, const double* gx, const double* gy,
                              const double* kp, const double* k0, cd* M) {
  const int n = 2 * nh;
  const int64_t nn = (int64_t)n * n, hh = (int64_t)nh * nh;
  const int64_t total = batch * nn;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / nn;
    const int rc = (int)(e % nn);
    const int r = rc / n, c = rc % n;
    const int i = r % nh, j = c % nh;
    const int bi = r / nh, bj = c / nh;
    const int64_t mo = (int64_t)map_index[b] * hh + (int64_t)i * nh + j;
    const double k = k0[b];
    const cd ax = mk(kp[4 * b + 0] / k, kp[4 * b + 1] / k), ay = mk(kp[4 * b + 2] / k, kp[4 * b + 3] / k);
    cd kxi, kyi;
    kvec(kp, k0, gx, gy, b, i, kxi, kyi);
    const bool dg = (i == j);
    const cd gxv = Hx[mo] * (1.0 / k) + (dg ? ax : mk(0.0));
    const cd gyv = Hy[mo] * (1.0 / k) + (dg ? ay : mk(0.0));
    cd v;
    if (bi == 0 && bj == 0) v = kxi * gxv - C[mo] + (dg ? kyi * kyi : mk(0.0));
    else if (bi == 0) v = kxi * gyv - (dg ? kxi * kyi : mk(0.0));
    else if (bj == 0) v = kyi * gxv - (dg ? kxi * kyi : mk(0.0));
    else v = kyi * gyv - C[mo] + (dg ? kxi * kxi : mk(0.0));
    M[e] = v;
  }
}

__global__ void k_sqrt_lam(int64_t count, cd* lam) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < count; e += (int64_t)gridDim.x * blockDim.x)
    lam[e] = csqrt(lam[e]);
}

// V = Q W / lam with Q = [[Kx Ky, C - Kx^2], [Ky^2 - C, -Kx Ky]] (alternative.py:167-176);
// CWt = C W_top, CWb = C W_bottom (nh x n each).
__global__ void k_modes_v(int64_t batch, int nh, const double* gx, const double* gy, const double* kp, const double* k0,
                          const cd* __restrict__ W, const cd* __restrict__ CWt, const cd* __restrict__ CWb,
                          const cd* __restrict__ lam, cd* V, int* status) {
  const int n = 2 * nh;
  const int64_t nn = (int64_t)n * n, hn = (int64_t)nh * n;
  const int64_t total = batch * nn;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / nn;
    const int rc = (int)(e % nn);
    const int r = rc / n, c = rc % n;
    const int i = r % nh;
    cd kx, ky;
    kvec(kp, k0, gx, gy, b, i, kx, ky);
    const cd wt = W[b * nn + (int64_t)i * n + c], wb = W[b * nn + (int64_t)(nh + i) * n + c];
    const cd kxy = kx * ky;
    cd q;
    if (r < nh) q = kxy * wt - kx * kx * wb + CWb[b * hn + (int64_t)i * n + c];
    else q = ky * ky * wt - CWt[b * hn + (int64_t)i * n + c] - kxy * wb;
    const cd l = lam[b * n + c];
    const cd v = cdiv(q, l);
    V[e] = v;
    if (!cfinite(v)) status_or(status, b, KHP_BIT_NONFINITE);
  }
}

// A = Wi + Vi V0, B = Wi - Vi V0 with V0 the free-space modes (per-harmonic 2x2).
__global__ void k_build_ab(int64_t batch, int nh, const double* gx, const double* gy, const double* kp,
                           const double* k0, const cd* __restrict__ Wi, const cd* __restrict__ Vi, cd* A, cd* B) {
  const int n = 2 * nh;
  const int64_t nn = (int64_t)n * n;
  const int64_t total = batch * nn;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / nn;
    const int rc = (int)(e % nn);
    const int r = rc / n, c = rc % n;
    const int g = c % nh, cb = c / nh;
    cd kx, ky;
    kvec(kp, k0, gx, gy, b, g, kx, ky);
    const cd one = mk(1.0);
    const cd kz0 = kz_branch(one - kx * kx - ky * ky);
    const cd il0 = cdiv(one, mk(-kz0.im, kz0.re));
    const M2 v0 = scale(il0, q_medium(kx, ky, one));
    const cd* vr = Vi + b * nn + (int64_t)r * n;
    const cd t2 = cb == 0 ? vr[g] * v0.a + vr[nh + g] * v0.c : vr[g] * v0.b + vr[nh + g] * v0.d;
    const cd w = Wi[e];
    A[e] = w + t2;
    B[e] = w - t2;
  }
}

__device__ __forceinline__ cd prop_x(const cd* lam, int64_t b, int n, int i, double dk) {
  return cexp(-(lam[b * n + i] * dk));
}

// M1 = X BAi X (in place), X = diag(exp(-lam k0 d)).
__global__ void k_xmx(int64_t batch, int n, const cd* __restrict__ lam, const double* depth, const double* k0, cd* M) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < batch * nn; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / nn;
    const int rc = (int)(e % nn);
    const double dk = depth[b] * k0[b];
    M[e] = prop_x(lam, b, n, rc / n, dk) * M[e] * prop_x(lam, b, n, rc % n, dk);
  }
}

// out[i][j] (leading dim ldo) = X_i in[i][j]
__global__ void k_xrows(int64_t batch, int n, const cd* __restrict__ lam, const double* depth, const double* k0,
                        const cd* __restrict__ in, cd* out, int64_t ldo, int64_t bso) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < batch * nn; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / nn;
    const int rc = (int)(e % nn);
    const int i = rc / n, j = rc % n;
    out[b * bso + (int64_t)i * ldo + j] = prop_x(lam, b, n, i, depth[b] * k0[b]) * in[e];
  }
}

// S = [[X1, X2], [X2, X1]] from the n x 2n solution [X1 | X2]
__global__ void k_scatter_sym(int64_t batch, int n, const cd* __restrict__ X, cd* S, int* status) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < batch * 2 * nn; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / (2 * nn);
    const int64_t rc = e % (2 * nn);
    const int i = (int)(rc / (2 * n)), jj = (int)(rc % (2 * n));
    const cd v = X[e];
    cd* Sb = S + b * 4 * nn;
    if (jj < n) {
      Sb[(int64_t)i * n + jj] = v;
      Sb[3 * nn + (int64_t)i * n + jj] = v;
    } else {
      Sb[nn + (int64_t)i * n + jj - n] = v;
      Sb[2 * nn + (int64_t)i * n + jj - n] = v;
    }
    if (!cfinite(v)) status_or(status, b, KHP_BIT_NONFINITE);
  }
}

// ------------------------------------------------------------------------------------------
// Fluxes: one CTA per problem.
// ------------------------------------------------------------------------------------------
__global__ void k_flux(int px, int py, const cd* __restrict__ S, int64_t s_stride, const double* gx, const double* gy,
                       const double* kp, const double* k0v, const cd* te_v, const cd* tm_v, cd epsi, cd epse,
                       double* R, double* T, double* r_orders, double* t_orders) {
  __shared__ TeamShared sh;
  TeamCta t;
  const int64_t b = blockIdx.x;
  const int nh = px * py, n = 2 * nh;
  const int64_t nn = (int64_t)n * n;
  const double k0 = k0v[b];
  const cd kpx = mk(kp[4 * b + 0], kp[4 * b + 1]), kpy = mk(kp[4 * b + 2], kp[4 * b + 3]);
  // incident plane wave and its polarisation (alternative.py:101-128)
  const cd kzi_abs = conj(csqrt(mk(k0 * k0) * epsi - kpx * kpx - kpy * kpy));
  const double kpn = sqrt(norm2(kpx) + norm2(kpy));
  const double kn = sqrt(norm2(kpx) + norm2(kpy) + norm2(kzi_abs));
  cd te = te_v[b], tm = tm_v[b];
  const double pn = hypot(cabs(te), cabs(tm));
  te = te * (1.0 / pn);
  tm = tm * (1.0 / pn);
  cd pol_x, pol_y;
  if (fabs(kpn) < 1e-8) {
    pol_x = te;
    pol_y = tm;
  } else {
    const cd bx = kpx * (1.0 / kn), by = kpy * (1.0 / kn), bz = kzi_abs * (1.0 / kn);
    // aTE = -(z_dev x kbar), z_dev = (0, 0, -1)  ->  (-by, bx, 0)
    cd ex = -by, ey = bx;
    const double ne = sqrt(norm2(ex) + norm2(ey));
    ex = ex * (1.0 / ne);
    ey = ey * (1.0 / ne);
    // aTM = aTE x kbar
    cd mx = ey * bz, my = -(ex * bz), mz = ex * by - ey * bx;
    const double nm = sqrt(norm2(mx) + norm2(my) + norm2(mz));
    mx = mx * (1.0 / nm);
    my = my * (1.0 / nm);
    pol_x = te * ex + tm * mx;
    pol_y = te * ey + tm * my;
  }
  const cd kzi_n = kzi_abs * (1.0 / k0);
  const int c0 = (nh - 1) / 2;
  const cd* S11 = S + b * s_stride;
  const cd* S21 = S11 + 2 * nn;
  double rs = 0.0, ts = 0.0;
  for (int g = t.tid(); g < nh; g += t.size()) {
    const cd kxa = mk(kp[4 * b + 0] + gx[g], kp[4 * b + 1]);
    const cd kya = mk(kp[4 * b + 2] + gy[g], kp[4 * b + 3]);
    const cd kx = kxa * (1.0 / k0), ky = kya * (1.0 / k0);
    const cd kzr = conj(csqrt(mk(k0 * k0) * conj(epsi) - kxa * kxa - kya * kya)) * (1.0 / k0);
    const cd kzt = conj(csqrt(mk(k0 * k0) * conj(epse) - kxa * kxa - kya * kya)) * (1.0 / k0);
    for (int which = 0; which < 2; ++which) {
      const cd* Sm = which == 0 ? S11 : S21;
      const cd kz = which == 0 ? kzr : kzt;
      const cd sx = Sm[(int64_t)g * n + c0] * pol_x + Sm[(int64_t)g * n + nh + c0] * pol_y;
      const cd sy = Sm[(int64_t)(nh + g) * n + c0] * pol_x + Sm[(int64_t)(nh + g) * n + nh + c0] * pol_y;
      const cd sz = -cdiv(kx * sx + ky * sy, kz);
      const double tg = kz.re / kzi_n.re * (norm2(sx) + norm2(sy) + norm2(sz));
      if (which == 0) {
        rs += tg;
        if (r_orders) r_orders[b * nh + g] = tg;
      } else {
        ts += tg;
        if (t_orders) t_orders[b * nh + g] = tg;
      }
    }
  }
  rs = team_sum(t, rs, &sh);
  ts = team_sum(t, ts, &sh);
  if (threadIdx.x == 0) {
    R[b] = rs;
    T[b] = ts;
  }
}

inline int ew_grid(int64_t total) { return (int)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, 152 * 32)); }

// ------------------------------------------------------------------------------------------
// Plans (workspace layout shared by sizing and execution)
// ------------------------------------------------------------------------------------------
struct PrepWs {
  cd* lu;
  cd* tmp;
  int* piv;
};
inline PrepWs plan_prep(Arena& a, int64_t nmaps, int nh) {
  PrepWs w;
  w.lu = a.take<cd>(nmaps * (size_t)nh * nh);
  w.tmp = a.take<cd>(nmaps * (size_t)nh * nh);
  w.piv = a.take<int>(nmaps * (size_t)nh);
  return w;
}

struct ModesWs {
  cd* M;
  cd* Z;
  cd* CWt;
  cd* CWb;
};
inline ModesWs plan_modes(Arena& a, int64_t batch, int nh) {
  const size_t n = 2 * (size_t)nh;
  ModesWs w;
  w.M = a.take<cd>(batch * n * n);
  w.Z = a.take<cd>(batch * n * n);
  w.CWt = a.take<cd>(batch * nh * n);
  w.CWb = a.take<cd>(batch * nh * n);
  return w;
}

struct SmatWs {
  cd *b0, *b1, *b2, *b3, *p1, *p2, *rhs, *tmp;
  int* piv;
};
inline SmatWs plan_smat(Arena& a, int64_t batch, int nh) {
  const size_t n = 2 * (size_t)nh, nn = n * n;
  SmatWs w;
  w.b0 = a.take<cd>(batch * nn);
  w.b1 = a.take<cd>(batch * nn);
  w.b2 = a.take<cd>(batch * nn);
  w.b3 = a.take<cd>(batch * nn);
  w.p1 = a.take<cd>(batch * nn);
  w.p2 = a.take<cd>(batch * nn);
  w.rhs = a.take<cd>(batch * 2 * nn);
  w.tmp = a.take<cd>(batch * nn);
  w.piv = a.take<int>(batch * n);
  return w;
}

struct StarWs {
  cd *D, *Y, *U;
  int* piv;
};
inline StarWs plan_star(Arena& a, int64_t batch, int n) {
  const size_t nn = (size_t)n * n;
  StarWs w;
  w.D = a.take<cd>(batch * nn);
  w.Y = a.take<cd>(batch * 2 * nn);
  w.U = a.take<cd>(batch * 2 * nn);
  w.piv = a.take<int>(batch * (size_t)n);
  return w;
}

struct ConvWs {
  cd* F;
};
inline ConvWs plan_conv(Arena& a, int64_t nmaps, int px, int py) {
  ConvWs w;
  w.F = a.take<cd>(nmaps * (size_t)(2 * px - 1) * (2 * py - 1));
  return w;
}

#define KHP_TRY(x)          \
  do {                      \
    const int _st = (x);    \
    if (_st) return _st;    \
  } while (0)

}  // namespace
}  // namespace khp

using namespace khp;

// ==========================================================================================
// C ABI
// ==========================================================================================
extern "C" {

int khp_version(void) { return 100; }

const char* khp_status_string(int code) {
  switch (code) {
    case KHP_OK: return "ok";
    case KHP_ERR_INVALID_ARG: return "invalid argument";
    case KHP_ERR_WORKSPACE: return "workspace too small";
    case KHP_ERR_CUDA: return "CUDA runtime error";
    case KHP_ERR_SINGULAR: return "singular matrix (zero pivot)";
    case KHP_ERR_NOT_CONVERGED: return "eigensolver did not converge";
    case KHP_ERR_NONFINITE: return "non-finite value (NaN/Inf), e.g. kz = 0 at a Wood anomaly";
    case KHP_ERR_TOO_LARGE: return "size exceeds the fixed capacity of this entry point";
    default: return "unknown status";
  }
}

size_t khp_convmat_workspace(int64_t nmaps, int32_t px, int32_t py) {
  Arena a{nullptr, 0};
  plan_conv(a, nmaps, px, py);
  return a.off;
}

int khp_convmat(int64_t nmaps, int64_t nx, int64_t ny, const double* eps, int32_t px, int32_t py, double* conv,
                void* workspace, size_t ws_bytes, void* stream) {
  if (nmaps < 0 || px < 1 || py < 1 || (px % 2) == 0 || (py % 2) == 0) return KHP_ERR_INVALID_ARG;
  if (nx < 2 * px - 1 || ny < 2 * py - 1 || ny > 8192 || !eps || !conv) return KHP_ERR_INVALID_ARG;
  if (nmaps == 0) return KHP_OK;
  Arena a{static_cast<char*>(workspace), ws_bytes};
  ConvWs w = plan_conv(a, nmaps, px, py);
  if (!a.ok || !workspace) return KHP_ERR_WORKSPACE;
  cudaStream_t s = as_stream(stream);
  const size_t smem = sizeof(cd) * (size_t)ny;
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute(k_convmat_dft, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return KHP_ERR_CUDA;
  k_convmat_dft<<<dim3(2 * px - 1, (unsigned)nmaps), 256, smem, s>>>(nx, ny, (const cd*)eps, px, py, w.F);
  count_launches(1);
  const int64_t total = nmaps * (int64_t)px * py * px * py;
  k_convmat_gather<<<ew_grid(total), 256, 0, s>>>(nmaps, px, py, w.F, (cd*)conv);
  count_launches(1);
  return cuda_status();
}

size_t khp_convmat_islands_workspace(int64_t nmaps, int32_t px, int32_t py) {
  Arena a{nullptr, 0};
  plan_conv(a, nmaps, px, py);
  return a.off;
}

int khp_convmat_islands(int64_t nmaps, int32_t px, int32_t py, int32_t nislands, const double* islands,
                        const double* eps_host, double b1x, double b1y, double b2x, double b2y, double cell_area,
                        double* conv, void* workspace, size_t ws_bytes, void* stream) {
  if (nmaps < 0 || px < 1 || py < 1 || (px % 2) == 0 || (py % 2) == 0 || nislands < 0 || !eps_host || !conv ||
      (nislands > 0 && !islands) || !(cell_area > 0.0))
    return KHP_ERR_INVALID_ARG;
  if (nmaps == 0) return KHP_OK;
  Arena a{static_cast<char*>(workspace), ws_bytes};
  ConvWs w = plan_conv(a, nmaps, px, py);
  if (!a.ok || !workspace) return KHP_ERR_WORKSPACE;
  cudaStream_t s = as_stream(stream);
  k_convmat_islands<<<ew_grid(nmaps * (int64_t)(2 * px - 1) * (2 * py - 1)), 256, 0, s>>>(
      nmaps, px, py, nislands, islands, (const cd*)eps_host, b1x, b1y, b2x, b2y, cell_area, w.F);
  count_launches(1);
  const int64_t total = nmaps * (int64_t)px * py * px * py;
  k_convmat_gather<<<ew_grid(total), 256, 0, s>>>(nmaps, px, py, w.F, (cd*)conv);
  count_launches(1);
  return cuda_status();
}

size_t khp_convmat_bwd_workspace(int64_t nmaps, int64_t ny, int32_t px, int32_t py) {
  if (nmaps < 0 || ny < 1 || px < 1 || py < 1) return 0;
  Arena a{nullptr, 0};
  a.take<cd>(nmaps * (size_t)(2 * px - 1) * (2 * py - 1));
  a.take<cd>(nmaps * (size_t)(2 * px - 1) * (size_t)ny);
  return a.off;
}

int khp_convmat_bwd(int64_t nmaps, int64_t nx, int64_t ny, const double* dconv, int32_t px, int32_t py, double* deps,
                    void* workspace, size_t ws_bytes, void* stream) {
  if (nmaps < 0 || px < 1 || py < 1 || (px % 2) == 0 || (py % 2) == 0) return KHP_ERR_INVALID_ARG;
  if (nx < 2 * px - 1 || ny < 2 * py - 1 || !dconv || !deps) return KHP_ERR_INVALID_ARG;
  if (nmaps == 0) return KHP_OK;
  Arena a{static_cast<char*>(workspace), ws_bytes};
  cd* dF = a.take<cd>(nmaps * (size_t)(2 * px - 1) * (2 * py - 1));
  cd* h = a.take<cd>(nmaps * (size_t)(2 * px - 1) * (size_t)ny);
  if (!a.ok || !workspace) return KHP_ERR_WORKSPACE;
  cudaStream_t s = as_stream(stream);
  k_convmat_bwd_gather<<<ew_grid(nmaps * (int64_t)(2 * px - 1) * (2 * py - 1)), 256, 0, s>>>(nmaps, px, py,
                                                                                            (const cd*)dconv, dF);
  count_launches(1);
  k_convmat_bwd_dft_y<<<ew_grid(nmaps * (int64_t)(2 * px - 1) * ny), 256, 0, s>>>(nmaps, px, py, ny, dF, h);
  count_launches(1);
  k_convmat_bwd_dft_x<<<ew_grid(nmaps * nx * ny), 256, 0, s>>>(nmaps, px, nx, ny, h, (cd*)deps);
  count_launches(1);
  return cuda_status();
}

size_t khp_structure_prep_workspace(int64_t nmaps, int32_t nh) {
  Arena a{nullptr, 0};
  plan_prep(a, nmaps, nh);
  return a.off;
}

int khp_structure_prep(int64_t nmaps, int32_t nh, const double* conv, const double* gx, const double* gy, double* ic,
                       double* hx, double* hy, int32_t* status, void* workspace, size_t ws_bytes, void* stream) {
  if (nmaps < 0 || nh < 1 || !conv || !gx || !gy || !ic || !hx || !hy || !status) return KHP_ERR_INVALID_ARG;
  if (nmaps == 0) return KHP_OK;
  Arena a{static_cast<char*>(workspace), ws_bytes};
  PrepWs w = plan_prep(a, nmaps, nh);
  if (!a.ok || !workspace) return KHP_ERR_WORKSPACE;
  cudaStream_t s = as_stream(stream);
  const int64_t hh = (int64_t)nh * nh;
  const cd* C = (const cd*)conv;
  KHP_TRY(launch_copy<double>(nmaps, nh, nh, C, nh, hh, w.lu, nh, hh, s));
  KHP_TRY(launch_inverse<double>(nmaps, nh, w.lu, nh, hh, (cd*)ic, nh, hh, w.piv, status, s));
  k_row_scale_real<<<ew_grid(nmaps * hh), 256, 0, s>>>(nmaps, nh, gx, C, w.tmp);
  count_launches(1);
  KHP_TRY(launch_gemm<double>(nmaps, nh, nh, nh, mk(1.0), (const cd*)ic, nh, hh, w.tmp, nh, hh, mk(0.0), (cd*)hx, nh,
                              hh, s));
  k_row_scale_real<<<ew_grid(nmaps * hh), 256, 0, s>>>(nmaps, nh, gy, C, w.tmp);
  count_launches(1);
  KHP_TRY(launch_gemm<double>(nmaps, nh, nh, nh, mk(1.0), (const cd*)ic, nh, hh, w.tmp, nh, hh, mk(0.0), (cd*)hy, nh,
                              hh, s));
  return cuda_status();
}

size_t khp_layer_modes_workspace(int64_t batch, int32_t nh) {
  Arena a{nullptr, 0};
  plan_modes(a, batch, nh);
  return a.off;
}

int khp_layer_modes(int64_t batch, int32_t nh, const int32_t* map_index, const double* conv, const double* hx,
                    const double* hy, const double* gx, const double* gy, const double* kp, const double* k0,
                    double* W, double* V, double* lam, int32_t* status, void* workspace, size_t ws_bytes,
                    void* stream) {
  if (batch < 0 || nh < 1 || !map_index || !conv || !hx || !hy || !gx || !gy || !kp || !k0 || !W || !V || !lam ||
      !status)
    return KHP_ERR_INVALID_ARG;
  if (batch == 0) return KHP_OK;
  Arena a{static_cast<char*>(workspace), ws_bytes};
  ModesWs w = plan_modes(a, batch, nh);
  if (!a.ok || !workspace) return KHP_ERR_WORKSPACE;
  cudaStream_t s = as_stream(stream);
  const int n = 2 * nh;
  const int64_t nn = (int64_t)n * n, hh = (int64_t)nh * nh, hn = (int64_t)nh * n;
  k_assemble_pq<<<ew_grid(batch * nn), 256, 0, s>>>(batch, nh, map_index, (const cd*)conv, (const cd*)hx,
                                                     (const cd*)hy, gx, gy, kp, k0, w.M);
  count_launches(1);
  KHP_TRY(cuda_status());
  KHP_TRY(launch_geev<double>(batch, n, w.M, n, nn, w.Z, (cd*)W, n, nn, (cd*)lam, n, status, s));
  k_sqrt_lam<<<ew_grid(batch * n), 256, 0, s>>>(batch * n, (cd*)lam);
  count_launches(1);
  KHP_TRY(launch_gemm<double>(batch, nh, n, nh, mk(1.0), (const cd*)conv, nh, hh, (const cd*)W, n, nn, mk(0.0), w.CWt,
                              n, hn, s, map_index));
  KHP_TRY(launch_gemm<double>(batch, nh, n, nh, mk(1.0), (const cd*)conv, nh, hh, (const cd*)W + hn, n, nn, mk(0.0),
                              w.CWb, n, hn, s, map_index));
  k_modes_v<<<ew_grid(batch * nn), 256, 0, s>>>(batch, nh, gx, gy, kp, k0, (const cd*)W, w.CWt, w.CWb,
                                                 (const cd*)lam, (cd*)V, status);
  count_launches(1);
  return cuda_status();
}

size_t khp_layer_smatrix_workspace(int64_t batch, int32_t nh) {
  Arena a{nullptr, 0};
  plan_smat(a, batch, nh);
  return a.off;
}

int khp_layer_smatrix(int64_t batch, int32_t nh, const double* W, const double* V, const double* lam,
                      const double* depth, const double* gx, const double* gy, const double* kp, const double* k0,
                      double* S, int32_t* status, void* workspace, size_t ws_bytes, void* stream) {
  if (batch < 0 || nh < 1 || !W || !V || !lam || !depth || !gx || !gy || !kp || !k0 || !S || !status)
    return KHP_ERR_INVALID_ARG;
  if (batch == 0) return KHP_OK;
  Arena a{static_cast<char*>(workspace), ws_bytes};
  SmatWs w = plan_smat(a, batch, nh);
  if (!a.ok || !workspace) return KHP_ERR_WORKSPACE;
  cudaStream_t s = as_stream(stream);
  const int n = 2 * nh;
  const int64_t nn = (int64_t)n * n;
  const cd one = mk(1.0), zero = mk(0.0), mone = mk(-1.0);
  const cd* L = (const cd*)lam;
  // t1 = W^-1 (W0 = I), t2 = V^-1 V0
  KHP_TRY(launch_copy<double>(batch, n, n, (const cd*)W, n, nn, w.b0, n, nn, s));
  KHP_TRY(launch_inverse<double>(batch, n, w.b0, n, nn, w.b2, n, nn, w.piv, status, s));  // b2 = Wi
  KHP_TRY(launch_copy<double>(batch, n, n, (const cd*)V, n, nn, w.b1, n, nn, s));
  KHP_TRY(launch_inverse<double>(batch, n, w.b1, n, nn, w.b3, n, nn, w.piv, status, s));  // b3 = Vi
  k_build_ab<<<ew_grid(batch * nn), 256, 0, s>>>(batch, nh, gx, gy, kp, k0, w.b2, w.b3, w.b0, w.b1);  // b0 = A, b1 = B
  KHP_TRY(cuda_status());
  count_launches(1);
  // Ai = A^-1 (b3 <- copy of A for the LU, b2 <- Ai)
  KHP_TRY(launch_copy<double>(batch, n, n, w.b0, n, nn, w.b3, n, nn, s));
  KHP_TRY(launch_inverse<double>(batch, n, w.b3, n, nn, w.b2, n, nn, w.piv, status, s));
  // p1 = X B Ai X
  KHP_TRY(launch_gemm<double>(batch, n, n, n, one, w.b1, n, nn, w.b2, n, nn, zero, w.p1, n, nn, s));
  k_xmx<<<ew_grid(batch * nn), 256, 0, s>>>(batch, n, L, depth, k0, w.p1);
  count_launches(1);
  // p2 = T = A - p1 B
  KHP_TRY(launch_copy<double>(batch, n, n, w.b0, n, nn, w.p2, n, nn, s));
  KHP_TRY(launch_gemm<double>(batch, n, n, n, mone, w.p1, n, nn, w.b1, n, nn, one, w.p2, n, nn, s));
  // rhs[:, :n] = p1 A - B
  KHP_TRY(launch_copy<double>(batch, n, n, w.b1, n, nn, w.rhs, 2 * n, 2 * nn, s));
  KHP_TRY(launch_gemm<double>(batch, n, n, n, one, w.p1, n, nn, w.b0, n, nn, mone, w.rhs, 2 * n, 2 * nn, s));
  // rhs[:, n:] = X (A - B Ai B)
  KHP_TRY(launch_gemm<double>(batch, n, n, n, one, w.b2, n, nn, w.b1, n, nn, zero, w.b3, n, nn, s));  // b3 = Ai B
  KHP_TRY(launch_copy<double>(batch, n, n, w.b0, n, nn, w.tmp, n, nn, s));
  KHP_TRY(launch_gemm<double>(batch, n, n, n, mone, w.b1, n, nn, w.b3, n, nn, one, w.tmp, n, nn, s));
  k_xrows<<<ew_grid(batch * nn), 256, 0, s>>>(batch, n, L, depth, k0, w.tmp, w.rhs + n, 2 * n, 2 * nn);
  count_launches(1);
  // [S11 | S12] = T^-1 rhs
  KHP_TRY(launch_getrf<double>(batch, n, w.p2, n, nn, w.piv, status, s));
  KHP_TRY(launch_getrs<double>(batch, n, w.p2, n, nn, w.piv, w.rhs, 2 * n, 2 * nn, 2 * n, s));
  k_scatter_sym<<<ew_grid(batch * 2 * nn), 256, 0, s>>>(batch, n, w.rhs, (cd*)S, status);
  count_launches(1);
  return cuda_status();
}

int khp_closed_form_smatrix(int64_t batch, int32_t nh, int32_t kind, const double* eps, const double* depth,
                            const double* gx, const double* gy, const double* kp, const double* k0, double* S,
                            double* W, double* V, double* lam, int32_t* status, void* stream) {
  if (batch < 0 || nh < 1 || kind < 0 || kind > 2 || !eps || !gx || !gy || !kp || !k0 || !S || !status)
    return KHP_ERR_INVALID_ARG;
  if (kind == 0 && !depth) return KHP_ERR_INVALID_ARG;
  if (batch == 0) return KHP_OK;
  cudaStream_t s = as_stream(stream);
  const int64_t n = 2 * (int64_t)nh, nn = n * n;
  if (cudaMemsetAsync(S, 0, sizeof(cd) * batch * 4 * nn, s) != cudaSuccess) return KHP_ERR_CUDA;
  if (W && cudaMemsetAsync(W, 0, sizeof(cd) * batch * nn, s) != cudaSuccess) return KHP_ERR_CUDA;
  if (V && cudaMemsetAsync(V, 0, sizeof(cd) * batch * nn, s) != cudaSuccess) return KHP_ERR_CUDA;
  k_closed_form<<<ew_grid(batch * nh), 256, 0, s>>>(batch, nh, kind, (const cd*)eps, depth, gx, gy, kp, k0, (cd*)S,
                                                     (cd*)W, (cd*)V, (cd*)lam, status);
  count_launches(1);
  return cuda_status();
}

size_t khp_star_product_workspace(int64_t batch, int32_t n) {
  Arena a{nullptr, 0};
  plan_star(a, batch, n);
  return a.off;
}

int khp_star_product(int64_t batch, int32_t n, const double* SA, int64_t sa_stride, const double* SB,
                     int64_t sb_stride, double* S, int32_t* status, void* workspace, size_t ws_bytes, void* stream) {
  if (batch < 0 || n < 1 || !SA || !SB || !S || !status || sa_stride < 0 || sb_stride < 0) return KHP_ERR_INVALID_ARG;
  if (batch == 0) return KHP_OK;
  Arena a{static_cast<char*>(workspace), ws_bytes};
  StarWs w = plan_star(a, batch, n);
  if (!a.ok || !workspace) return KHP_ERR_WORKSPACE;
  cudaStream_t s = as_stream(stream);
  const int64_t nn = (int64_t)n * n;
  const cd one = mk(1.0), zero = mk(0.0), mone = mk(-1.0);
  const cd* A = (const cd*)SA;
  const cd* B = (const cd*)SB;
  cd* O = (cd*)S;
  const cd *A11 = A, *A12 = A + nn, *A21 = A + 2 * nn, *A22 = A + 3 * nn;
  const cd *B11 = B, *B12 = B + nn, *B21 = B + 2 * nn, *B22 = B + 3 * nn;
  const int64_t os = 4 * nn;
  // D = I - SB11 SA22
  KHP_TRY(launch_identity<double>(batch, n, n, w.D, n, nn, one, s));
  KHP_TRY(launch_gemm<double>(batch, n, n, n, mone, B11, n, sb_stride, A22, n, sa_stride, one, w.D, n, nn, s));
  KHP_TRY(launch_getrf<double>(batch, n, w.D, n, nn, w.piv, status, s));
  // Y = D^-1 [SB11 SA21 | SB12]
  KHP_TRY(launch_gemm<double>(batch, n, n, n, one, B11, n, sb_stride, A21, n, sa_stride, zero, w.Y, 2 * n, 2 * nn, s));
  KHP_TRY(launch_copy<double>(batch, n, n, B12, n, sb_stride, w.Y + n, 2 * n, 2 * nn, s));
  KHP_TRY(launch_getrs<double>(batch, n, w.D, n, nn, w.piv, w.Y, 2 * n, 2 * nn, 2 * n, s));
  // S11 = SA11 + SA12 Y1 ; S12 = SA12 Y2
  KHP_TRY(launch_copy<double>(batch, n, n, A11, n, sa_stride, O, n, os, s));
  KHP_TRY(launch_gemm<double>(batch, n, n, n, one, A12, n, sa_stride, w.Y, 2 * n, 2 * nn, one, O, n, os, s));
  KHP_TRY(launch_gemm<double>(batch, n, n, n, one, A12, n, sa_stride, w.Y + n, 2 * n, 2 * nn, zero, O + nn, n, os, s));
  // U = SA22 Y ; U1 += SA21
  KHP_TRY(launch_gemm<double>(batch, n, 2 * n, n, one, A22, n, sa_stride, w.Y, 2 * n, 2 * nn, zero, w.U, 2 * n,
                              2 * nn, s));
  KHP_TRY(launch_axpby<double>(batch, n, n, one, w.U, 2 * n, 2 * nn, one, A21, n, sa_stride, w.U, 2 * n, 2 * nn, s));
  // S21 = SB21 U1 ; S22 = SB22 + SB21 U2
  KHP_TRY(launch_gemm<double>(batch, n, n, n, one, B21, n, sb_stride, w.U, 2 * n, 2 * nn, zero, O + 2 * nn, n, os, s));
  KHP_TRY(launch_copy<double>(batch, n, n, B22, n, sb_stride, O + 3 * nn, n, os, s));
  KHP_TRY(launch_gemm<double>(batch, n, n, n, one, B21, n, sb_stride, w.U + n, 2 * n, 2 * nn, one, O + 3 * nn, n, os,
                              s));
  return cuda_status();
}

int khp_flux(int64_t batch, int32_t px, int32_t py, const double* S, int64_t s_stride, const double* gx,
             const double* gy, const double* kp, const double* k0, const double* te, const double* tm, double epsi_re,
             double epsi_im, double epse_re, double epse_im, double* R, double* T, double* r_orders, double* t_orders,
             void* stream) {
  if (batch < 0 || px < 1 || py < 1 || !S || !gx || !gy || !kp || !k0 || !te || !tm || !R || !T || s_stride < 0)
    return KHP_ERR_INVALID_ARG;
  if (batch == 0) return KHP_OK;
  k_flux<<<(unsigned)batch, 128, 0, as_stream(stream)>>>(px, py, (const cd*)S, s_stride, gx, gy, kp, k0,
                                                         (const cd*)te, (const cd*)tm, mk(epsi_re, epsi_im),
                                                         mk(epse_re, epse_im), R, T, r_orders, t_orders);
  count_launches(1);
  return cuda_status();
}

}  // extern "C"
