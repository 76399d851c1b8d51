// Plane-wave amplitudes of a beam sampled over a Brillouin-zone-integration supercell
// (khepri/beams.py:164-190, amplitudes_from_fields; the DFT is fourier.slow_dft,
// khepri/fourier.py:94-104).
//
// The reference divides the sampled fields by the incident phase exp(i kp.r), cuts the
// [X][Y] sample grid into bzs[0] x bzs[1] cells of ns x ns points, and sums over the cells the
// direct DFT of the four transverse components (Ex, Ey, Hx, Hy) at the expansion's g vectors,
// divided by (cells * ns).  Its cutting pairs the field samples of cell i with the coordinates of
// another cell when the cell grid is not symmetric (np.split along different axes for the
// fields, which are then swapped, and for x, y, which are not); the index maps below reproduce
// that pairing exactly:
//   cell i, point (ix, iy):  field sample  (c1 ns + ix, c0 ns + iy), c0 = i / bzs1, c1 = i % bzs1
//                            coordinates   (d1 ns + ix, d0 ns + iy), d1 = i / bzs0, d0 = i % bzs0
// Pass 1 (thread per point) divides by the phase and gathers the coordinates; pass 2 (CTA per
// g vector) reduces the DFT sums in FP64.
#include <cuda_runtime.h>

#include <algorithm>

#include "khepri_gb300.h"
#include "khp_core.cuh"
#include "khp_launch.h"

namespace khp {
namespace {

using cd = cplx<double>;

__global__ void k_bzi_gather(int bzs0, int bzs1, int ns, const cd* __restrict__ fields, const double* __restrict__ x,
                             const double* __restrict__ y, const cd* __restrict__ kp, cd* __restrict__ fdiv,
                             double* __restrict__ xc, double* __restrict__ yc) {
  const cd kx = kp[0], ky = kp[1];
  const int64_t npts = (int64_t)bzs0 * bzs1 * ns * ns;
  const int64_t Y = (int64_t)bzs0 * ns;  // second axis of the sample grid
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < npts; p += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = p / ((int64_t)ns * ns);
    const int ix = (int)((p / ns) % ns), iy = (int)(p % ns);
    const int c0 = (int)(i / bzs1), c1 = (int)(i % bzs1);
    const int d1 = (int)(i / bzs0), d0 = (int)(i % bzs0);
    const int64_t sf = (int64_t)(c1 * ns + ix) * Y + (c0 * ns + iy);  // field sample
    const int64_t sc = (int64_t)(d1 * ns + ix) * Y + (d0 * ns + iy);  // paired coordinates
    // 1 / exp(i (kx x + ky y)) at the field sample's own position
    const cd arg = kx * x[sf] + ky * y[sf];  // complex for a complex kp
    const double mag = exp(arg.im);           // |exp(-i arg)| = exp(Im arg)
    double sn, cs;
    sincos(arg.re, &sn, &cs);
    const cd inv = mk(mag * cs, -mag * sn);
    const cd* f = fields + sf * 6;  // [2 (E, H)][3 (x, y, z)]
    fdiv[p * 4 + 0] = f[0] * inv;
    fdiv[p * 4 + 1] = f[1] * inv;
    fdiv[p * 4 + 2] = f[3] * inv;
    fdiv[p * 4 + 3] = f[4] * inv;
    xc[p] = x[sc];
    yc[p] = y[sc];
  }
}

__global__ void __launch_bounds__(256) k_bzi_dft(int64_t npts, const cd* __restrict__ fdiv, const double* __restrict__ xc,
                                                 const double* __restrict__ yc, const double* __restrict__ gx,
                                                 const double* __restrict__ gy, int ng, double scale, cd* out) {
  __shared__ double red[8][8];  // [warp][component re/im]
  const int g = blockIdx.x;
  const double kx = gx[g], ky = gy[g];
  double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int64_t p = threadIdx.x; p < npts; p += blockDim.x) {
    double sn, cs;
    sincos(kx * xc[p] + ky * yc[p], &sn, &cs);
    const cd e = mk(cs, -sn);  // exp(-i (kx x + ky y))
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const cd v = fdiv[p * 4 + j] * e;
      acc[2 * j] += v.re;
      acc[2 * j + 1] += v.im;
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    double v = acc[q];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp][q] = v;
  }
  __syncthreads();
  if (threadIdx.x < 8) {
    double v = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += red[w][threadIdx.x];
    const int j = threadIdx.x >> 1;
    double* o = reinterpret_cast<double*>(out + (int64_t)j * ng + g);
    o[threadIdx.x & 1] = v * scale;
  }
}

}  // namespace
}  // namespace khp

using namespace khp;

extern "C" {

size_t khp_bzi_amplitudes_workspace(int32_t bzs0, int32_t bzs1, int32_t ns) {
  if (bzs0 < 1 || bzs1 < 1 || ns < 1) return 0;
  const size_t npts = (size_t)bzs0 * bzs1 * ns * ns;
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  return al(npts * 4 * sizeof(cd)) + 2 * al(npts * sizeof(double));
}

int khp_bzi_amplitudes(int32_t bzs0, int32_t bzs1, int32_t ns, const double* fields, const double* x, const double* y,
                       const double* kp, int32_t ng, const double* gx, const double* gy, double* out, void* workspace,
                       size_t ws_bytes, void* stream) {
  if (bzs0 < 1 || bzs1 < 1 || ns < 1 || ng < 1 || !fields || !x || !y || !kp || !gx || !gy || !out)
    return KHP_ERR_INVALID_ARG;
  const size_t need = khp_bzi_amplitudes_workspace(bzs0, bzs1, ns);
  if (!workspace || ws_bytes < need) return KHP_ERR_WORKSPACE;
  const int64_t npts = (int64_t)bzs0 * bzs1 * ns * ns;
  auto al = [](size_t v) { return (v + 255) & ~size_t(255); };
  char* base = static_cast<char*>(workspace);
  cd* fdiv = reinterpret_cast<cd*>(base);
  double* xc = reinterpret_cast<double*>(base + al(npts * 4 * sizeof(cd)));
  double* yc = reinterpret_cast<double*>(base + al(npts * 4 * sizeof(cd)) + al(npts * sizeof(double)));
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>((npts + 255) / 256, 152 * 32));
  k_bzi_gather<<<blocks, 256, 0, s>>>(bzs0, bzs1, ns, reinterpret_cast<const cd*>(fields), x, y,
                                      reinterpret_cast<const cd*>(kp), fdiv, xc, yc);
  count_launches(1);
  if (cuda_status()) return KHP_ERR_CUDA;
  const double scale = 1.0 / ((double)bzs0 * bzs1 * ns);
  k_bzi_dft<<<(unsigned)ng, 256, 0, s>>>(npts, fdiv, xc, yc, gx, gy, ng, scale, reinterpret_cast<cd*>(out));
  count_launches(1);
  return cuda_status();
}

}  // extern "C"
