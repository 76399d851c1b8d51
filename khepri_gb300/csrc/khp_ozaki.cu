// FP64-accurate complex matrix products on the tensor cores (Ozaki's error-free splitting).
//
// GB300 runs FP64 at ~1.2 TFLOP/s and bf16 tensor-core products at over a hundred times that.
// C = A B with FP64 complex operands is formed here as a sum of bf16 x bf16 products that are
// exact in the FP32 accumulators:
//   1. every row of A and every column of B is scaled by a power of two into [-1, 1) and cut into
//      kDig = 7 signed 8-bit digits, q_i = rint(r 2^(8(i+1))), r -= q_i 2^-(8(i+1));
//      |q_0| <= 256 and |q_i| <= 128 are integers, exact in bf16, and the remainder after seven
//      digits is at most 2^-57;
//   2. the complex product becomes one real product [Re A | Im A] [[Re B, Im B], [-Im B, Re B]]
//      of inner size 2k and 2n columns ([Re C | Im C]);
//   3. the digit pairs (i, j) with i + j = l < kDig (28 pairs) are accumulated level by level with
//      mma.sync m16n8k16 (bf16 in, FP32 accumulate).  Over one 64-wide slice of the inner index
//      every partial sum of a level is an integer below 2.25 * 2^22 < 2^24, hence exact; the
//      slices are summed in int32 and each level is added to the FP64 result once, scaled by
//      2^-(8(l+2)).
// Error: ~2^-55 * 2k * (row max of A) * (column max of B) per element, the size of an FP64
// product's own rounding bound (the dropped pairs, i + j >= 7, are below that).
//
// Layout of the digit arrays (bf16, zero-padded so that the product kernel has no bounds checks):
//   Ad [problem][digit][Mp][K2p]   rows of [Re A | Im A]; row exponents ea [problem][Mp]
//   Bd [problem][digit][N2p][K2p]  columns of the real-ified B, inner index contiguous;
//                                  column exponents eb [problem][n] (shared by Re and Im columns)
// Mp, N2p, K2p: m, 2n, 2k rounded up to 64.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "khepri_gb300.h"
#include "khp_core.cuh"
#include "khp_launch.h"

namespace khp {
namespace {

using cd = cplx<double>;
using bf16 = __nv_bfloat16;

constexpr int kDig = 7;
constexpr int kT = 64;  // tile rows, tile columns and inner slice

inline int up64(int x) { return (x + 63) & ~63; }

// Biased binary exponent of x with subnormals counted as 1 (0 for x == 0, 2047 for inf / NaN).
__device__ __forceinline__ int biased_exp(double x) {
  const uint64_t u = (uint64_t)__double_as_longlong(x);
  const int be = (int)((u >> 52) & 0x7ff);
  return be == 0 ? ((u << 1) != 0 ? 1 : 0) : be;
}

// Scale exponent of a row / column from its largest biased exponent: every |x| < 2^e.
__device__ __forceinline__ int scale_exp(int bemax) { return bemax > 0 ? bemax - 1022 : 0; }

// Digits of x 2^-e (|x| < 2^e) into out[i * dstride], integer arithmetic only: X = round(x 2^(56-e))
// (|X| < 2^56, error <= 2^(e-57)) is cut into balanced base-256 digits, q_6 .. q_1 in [-128, 127]
// from the low end, q_0 = the rest (|q_0| <= 256).  inf / NaN yield a NaN digit.
__device__ __forceinline__ void put_digits(double x, int e, bf16* out, int64_t dstride) {
  const uint64_t u = (uint64_t)__double_as_longlong(x);
  const int be = (int)((u >> 52) & 0x7ff);
  if (be == 0x7ff) {
    out[0] = __float2bfloat16_rn(__int_as_float(0x7fc00000));
#pragma unroll
    for (int i = 1; i < kDig; ++i) out[i * dstride] = __float2bfloat16_rn(0.f);
    return;
  }
  const uint64_t frac = u & 0xfffffffffffffull;
  const uint64_t mant = be == 0 ? frac : (frac | (1ull << 52));
  // x = mant 2^(max(be, 1) - 1075), so X = mant 2^sh with sh <= 3 because |x| < 2^e
  const int sh = (be == 0 ? 1 : be) - 1075 + 56 - e;
  uint64_t mag;
  if (sh >= 0)
    mag = mant << sh;
  else if (sh > -63)
    mag = (mant + (1ull << (-sh - 1))) >> (-sh);
  else
    mag = 0;
  int64_t X = (u >> 63) ? -(int64_t)mag : (int64_t)mag;
#pragma unroll
  for (int i = kDig - 1; i >= 1; --i) {
    const int q = (int)((X + 128) & 255) - 128;
    X = (X - q) >> 8;  // exact
    out[i * dstride] = __int2bfloat16_rn(q);
  }
  out[0] = __int2bfloat16_rn((int)X);
}

__device__ __forceinline__ int warp_max(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// A digits, one warp per (problem, padded row); aidx (optional): problem b takes A[aidx[b]].
__global__ void k_split_a(int64_t batch, int m, int k, const cd* __restrict__ A, int64_t lda, int64_t bsA,
                          const int* __restrict__ aidx, int Mp, int K2p, bf16* __restrict__ Ad, int* __restrict__ ea) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; w < batch * Mp; w += nwarps) {
    const int64_t b = w / Mp;
    const int r = (int)(w % Mp);
    const bool live = r < m;
    const cd* row = A + (aidx ? (int64_t)aidx[b] : b) * bsA + (int64_t)r * lda;
    int bm = 0;
    if (live)
      for (int kk = lane; kk < k; kk += 32) bm = max(bm, max(biased_exp(row[kk].re), biased_exp(row[kk].im)));
    const int ex = scale_exp(warp_max(bm));
    if (lane == 0) ea[w] = ex;
    const int64_t ds = (int64_t)Mp * K2p;
    bf16* base = Ad + b * kDig * ds + (int64_t)r * K2p;
    for (int kk = lane; kk < K2p; kk += 32) {
      double x = 0.0;
      if (live) x = kk < k ? row[kk].re : (kk < 2 * k ? row[kk - k].im : 0.0);
      put_digits(x, ex, base + kk, ds);
    }
  }
}

// Column exponents of B, one thread per (problem, column).
__global__ void k_col_exp(int64_t batch, int k, int n, const cd* __restrict__ B, int64_t ldb, int64_t bsB,
                          int* __restrict__ eb) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < batch * n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / n;
    const int c = (int)(e % n);
    const cd* col = B + b * bsB + c;
    int bm = 0;
    for (int kk = 0; kk < k; ++kk) {
      const cd v = col[(int64_t)kk * ldb];
      bm = max(bm, max(biased_exp(v.re), biased_exp(v.im)));
    }
    eb[e] = scale_exp(bm);
  }
}

// B digits through a shared-memory transpose: block (32, 8) covers 32 real columns j x 32 inner
// indices kk of one problem; the values are gathered along j (coalesced reads of B's rows) and
// the digits written along kk (coalesced).  Real column j < n: [Re B; -Im B] of column j;
// n <= j < 2n: [Im B; Re B] of column j - n; zero outside 2n x 2k.
__global__ void __launch_bounds__(256) k_split_b(int k, int n, const cd* __restrict__ B, int64_t ldb, int64_t bsB,
                                                 int N2p, int K2p, const int* __restrict__ eb, bf16* __restrict__ Bd) {
  __shared__ double xs[32][33];
  const int64_t b = blockIdx.z;
  const int j0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const cd* Bb = B + b * bsB;
  {
    const int j = j0 + tx;
    const int c = j < n ? j : j - n;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int kl = ty + 8 * i;
      const int kk = k0 + kl;
      double x = 0.0;
      if (j < 2 * n && kk < 2 * k) {
        const cd v = Bb[(int64_t)(kk < k ? kk : kk - k) * ldb + c];
        x = j < n ? (kk < k ? v.re : -v.im) : (kk < k ? v.im : v.re);
      }
      xs[kl][tx] = x;
    }
  }
  __syncthreads();
  const int64_t per = (int64_t)N2p * K2p;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int jl = ty + 8 * i;
    const int j = j0 + jl;
    const int ex = j < 2 * n ? eb[b * n + (j < n ? j : j - n)] : 0;
    put_digits(xs[tx][jl], ex, Bd + b * kDig * per + (int64_t)j * K2p + k0 + tx, per);
  }
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(src));
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

__device__ __forceinline__ void ldsm_x4(uint32_t addr, uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(addr));
}

__device__ __forceinline__ void mma_bf16(float* d, const uint32_t* a, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Byte offset of 16-byte chunk ch of row r in a 64 x 64 bf16 tile (128-byte rows), XOR-swizzled
// so that the eight rows read by one ldmatrix phase fall in eight different bank groups.
__device__ __forceinline__ uint32_t swz(int r, int ch) { return (uint32_t)(r * 128 + ((ch ^ (r & 7)) << 4)); }

// Stage sequence of the product: for every level l, every 64-wide inner slice kc, the digit pairs
// (da, l - da), da = 0 .. l.
struct Stage {
  int lvl, kc, da;
  __device__ __forceinline__ void next(int K2p) {
    if (++da > lvl) {
      da = 0;
      kc += kT;
      if (kc >= K2p) {
        kc = 0;
        ++lvl;
      }
    }
  }
};

constexpr int kStages = 4;                  // cp.async pipeline depth
constexpr int kTileBytes = kT * kT * 2;     // one 64 x 64 bf16 tile
constexpr int kStageBytes = 2 * kTileBytes;  // A and B tiles
constexpr int kGemmSmem = kStages * kStageBytes;

// One 64 x 64 tile of the real output [Re C | Im C] per CTA (grid: N2p/64, Mp/64, problems);
// 4 warps of 32 x 32.  The A and B tiles of each stage are staged in shared memory by cp.async,
// kStages deep.
__global__ void __launch_bounds__(128) k_ozaki_gemm(int m, int n, int Mp, int N2p, int K2p, const bf16* __restrict__ Ad,
                                                    const int* __restrict__ ea, const bf16* __restrict__ Bd,
                                                    const int* __restrict__ eb, cd* C, int64_t ldc, int64_t bsC,
                                                    int64_t boff) {
  extern __shared__ __align__(128) unsigned char sm[];
  const int64_t b = blockIdx.z + boff;
  const int64_t dsA = (int64_t)Mp * K2p, dsB = (int64_t)N2p * K2p;
  const bf16* A0 = Ad + b * kDig * dsA + (int64_t)blockIdx.y * kT * K2p;
  const bf16* B0 = Bd + b * kDig * dsB + (int64_t)blockIdx.x * kT * K2p;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int wm = warp >> 1, wn = warp & 1;
  const uint32_t sbase = smem_addr(sm);
  const int nstages = kDig * (kDig + 1) / 2 * (K2p / kT);

  auto load = [&](int slot, const Stage& st) {
    const bf16* a = A0 + st.da * dsA + st.kc;
    const bf16* bb = B0 + (st.lvl - st.da) * dsB + st.kc;
    const uint32_t sa = sbase + slot * kStageBytes, sb = sa + kTileBytes;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int c = tid + i * 128;
      const int r = c >> 3, ch = c & 7;
      cp_async16(sa + swz(r, ch), a + (int64_t)r * K2p + ch * 8);
      cp_async16(sb + swz(r, ch), bb + (int64_t)r * K2p + ch * 8);
    }
  };

  double acc[2][4][4];
  int lsum[2][4][4];
  float part[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        acc[i][j][q] = 0.0;
        lsum[i][j][q] = 0;
        part[i][j][q] = 0.f;
      }

  Stage ld{0, 0, 0}, cs{0, 0, 0};
#pragma unroll
  for (int i = 0; i < kStages - 1; ++i) {
    if (i < nstages) {
      load(i, ld);
      ld.next(K2p);
    }
    cp_commit();
  }
  for (int it = 0; it < nstages; ++it) {
    cp_wait<kStages - 2>();  // stage it has landed (this thread's copies) ...
    __syncthreads();         // ... for every thread; the slot refilled below was read at it - 1
    if (it + kStages - 1 < nstages) {
      load((it + kStages - 1) % kStages, ld);
      ld.next(K2p);
    }
    cp_commit();
    const uint32_t sa = sbase + (it % kStages) * kStageBytes, sb = sa + kTileBytes;
    const int j = lane >> 3;
#pragma unroll
    for (int ks = 0; ks < kT / 16; ++ks) {
      uint32_t af[2][4], bfr[4][2];
#pragma unroll
      for (int mt = 0; mt < 2; ++mt) {
        const int r = wm * 32 + mt * 16 + (j & 1) * 8 + (lane & 7);
        ldsm_x4(sa + swz(r, ks * 2 + (j >> 1)), af[mt][0], af[mt][1], af[mt][2], af[mt][3]);
      }
#pragma unroll
      for (int np = 0; np < 2; ++np) {
        const int r = wn * 32 + np * 16 + (j >> 1) * 8 + (lane & 7);
        ldsm_x4(sb + swz(r, ks * 2 + (j & 1)), bfr[2 * np][0], bfr[2 * np][1], bfr[2 * np + 1][0],
                bfr[2 * np + 1][1]);
      }
#pragma unroll
      for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) mma_bf16(part[mt][nt], af[mt], bfr[nt][0], bfr[nt][1]);
    }
    if (cs.da == cs.lvl) {
      // the slice's pairs of this level are complete: its exact FP32 sum joins the level's int32 sum
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int jj = 0; jj < 4; ++jj)
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            lsum[i][jj][q] += __float2int_rn(part[i][jj][q]);
            part[i][jj][q] = 0.f;
          }
      if (cs.kc + kT >= K2p) {
        const double scale = ldexp(1.0, -8 * (cs.lvl + 2));
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
          for (int jj = 0; jj < 4; ++jj)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              acc[i][jj][q] = fma((double)lsum[i][jj][q], scale, acc[i][jj][q]);
              lsum[i][jj][q] = 0;
            }
      }
    }
    cs.next(K2p);
  }
  cp_wait<0>();

  const int g = lane >> 2, t4 = lane & 3;
  const int* EA = ea + b * Mp;
  const int* EB = eb + b * n;
  cd* Cb = C + b * bsC;
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int nt = 0; nt < 4; ++nt)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int r = blockIdx.y * kT + wm * 32 + mt * 16 + g + (q >= 2 ? 8 : 0);
        const int c = blockIdx.x * kT + wn * 32 + nt * 8 + t4 * 2 + (q & 1);
        if (r >= m || c >= 2 * n) continue;
        const int cc = c < n ? c : c - n;
        const double v = ldexp(acc[mt][nt][q], EA[r] + EB[cc]);
        if (c < n)
          Cb[(int64_t)r * ldc + cc].re = v;
        else
          Cb[(int64_t)r * ldc + cc].im = v;
      }
}

inline unsigned grid_of(int64_t total, int threads) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((total + threads - 1) / threads, 152 * 32));
}

int split_a(int64_t batch, int m, int k, const cd* A, int64_t lda, int64_t bsA, const int* aidx, void* Ad, int* ea,
            cudaStream_t s) {
  const int Mp = up64(m);
  k_split_a<<<grid_of(batch * Mp * 32, 256), 256, 0, s>>>(batch, m, k, A, lda, bsA, aidx, Mp, up64(2 * k),
                                                           static_cast<bf16*>(Ad), ea);
  count_launches(1);
  return cuda_status();
}

int split_b(int64_t batch, int k, int n, const cd* B, int64_t ldb, int64_t bsB, void* Bd, int* eb, cudaStream_t s) {
  const int N2p = up64(2 * n), K2p = up64(2 * k);
  k_col_exp<<<grid_of(batch * n, 128), 128, 0, s>>>(batch, k, n, B, ldb, bsB, eb);
  count_launches(1);
  for (int64_t off = 0; off < batch; off += 65535) {
    const unsigned nb = (unsigned)std::min<int64_t>(batch - off, 65535);
    k_split_b<<<dim3(N2p / 32, K2p / 32, nb), dim3(32, 8), 0, s>>>(k, n, B + off * bsB, ldb, bsB, N2p, K2p,
                                                                   eb + off * n, static_cast<bf16*>(Bd) + off * kDig * (int64_t)N2p * K2p);
    count_launches(1);
  }
  return cuda_status();
}

int product(int64_t batch, int m, int n, int k, const void* Ad, const int* ea, const void* Bd, const int* eb, cd* C,
            int64_t ldc, int64_t bsC, cudaStream_t s) {
  // dynamic shared memory above 48 KB is an opt-in per device (cheap to repeat)
  if (cudaFuncSetAttribute(k_ozaki_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, kGemmSmem) != cudaSuccess)
    return KHP_ERR_CUDA;
  const int Mp = up64(m), N2p = up64(2 * n), K2p = up64(2 * k);
  for (int64_t off = 0; off < batch; off += 65535) {
    const unsigned nb = (unsigned)std::min<int64_t>(batch - off, 65535);
    const dim3 grid(N2p / kT, Mp / kT, nb);
    k_ozaki_gemm<<<grid, 128, kGemmSmem, s>>>(m, n, Mp, N2p, K2p, static_cast<const bf16*>(Ad), ea,
                                      static_cast<const bf16*>(Bd), eb, C, ldc, bsC, off);
    count_launches(1);
  }
  return cuda_status();
}

}  // namespace

size_t ozaki_a_elems(int m, int k) { return std::max((size_t)kDig * up64(m) * up64(2 * k), tc_a_elems(8, m, k)); }
size_t ozaki_b_elems(int k, int n) { return std::max((size_t)kDig * up64(2 * n) * up64(2 * k), tc_b_elems(8, k, n)); }
int ozaki_rows_padded(int m) { return std::max(up64(m), tc_rows_padded(m)); }

int64_t ozaki_chunk(int64_t batch) {
  const int64_t parts = (batch + kOzakiMaxChunk - 1) / kOzakiMaxChunk;
  return parts > 0 ? (batch + parts - 1) / parts : 0;
}

int ozaki_zgemm(int64_t batch, int m, int n, int k, const cplx<double>* A, int64_t lda, int64_t bsA, const int* aidx,
                const cplx<double>* B, int64_t ldb, int64_t bsB, cplx<double>* C, int64_t ldc, int64_t bsC,
                const OzakiWs& w, cudaStream_t s, int digits) {
  if (batch <= 0 || m <= 0 || n <= 0) return KHP_OK;
  // the int32 level sums stay below 2.25 * 2^16 * K2p, under 2^31 for k <= 4096
  if (k <= 0 || k > 4096) return KHP_ERR_INVALID_ARG;
  // tcgen05 with TMEM level accumulators where its exactness bound and the scratch allow
  if (w.err && up64(2 * k) <= tc_max_k2p(8) && w.ad_elems >= tc_a_elems(8, m, k) &&
      w.bd_elems >= tc_b_elems(8, k, n) && w.ea_n >= (size_t)tc_rows_padded(m) && w.eb_n >= (size_t)n) {
    if (digits == 6)
      return tc_product<6, double, double>(batch, m, n, k, A, lda, bsA, aidx, B, ldb, bsB, nullptr, mk(1.0), mk(0.0),
                                           C, ldc, bsC, w, s);
    return tc_product<8, double, double>(batch, m, n, k, A, lda, bsA, aidx, B, ldb, bsB, nullptr, mk(1.0), mk(0.0), C,
                                         ldc, bsC, w, s);
  }
  const int64_t per_a = (int64_t)kDig * up64(m) * up64(2 * k), per_b = (int64_t)kDig * up64(2 * n) * up64(2 * k);
  const int64_t cap = std::min(std::min<int64_t>((int64_t)(w.ad_elems / per_a), (int64_t)(w.ea_n / up64(m))),
                               std::min<int64_t>((int64_t)(w.bd_elems / per_b), (int64_t)(w.eb_n / n)));
  const int64_t chunk = std::min(cap, ozaki_chunk(batch));
  if (chunk <= 0) return KHP_ERR_WORKSPACE;
  stage_begin(KHP_STAGE_TC_PRODUCT, s);
  for (int64_t off = 0; off < batch; off += chunk) {
    const int64_t nb = std::min<int64_t>(chunk, batch - off);
    int st = aidx ? split_a(nb, m, k, A, lda, bsA, aidx + off, w.ad, w.ea, s)
                  : split_a(nb, m, k, A + off * bsA, lda, bsA, nullptr, w.ad, w.ea, s);
    if (!st) st = split_b(nb, k, n, B + off * bsB, ldb, bsB, w.bd, w.eb, s);
    if (!st) st = product(nb, m, n, k, w.ad, w.ea, w.bd, w.eb, C + off * bsC, ldc, bsC, s);
    if (st) return st;
  }
  stage_end(KHP_STAGE_TC_PRODUCT, s);
  return KHP_OK;
}

}  // namespace khp

using namespace khp;

namespace {

struct WsLayout {
  size_t ad, ea, bd, eb, err, total;
};

WsLayout abi_layout(int64_t chunk, int m, int n, int k) {
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  WsLayout l;
  l.ad = 0;
  l.ea = l.ad + al((size_t)chunk * ozaki_a_elems(m, k) * 2);
  l.bd = l.ea + al((size_t)chunk * ozaki_rows_padded(m) * sizeof(int));
  l.eb = l.bd + al((size_t)chunk * ozaki_b_elems(k, n) * 2);
  l.err = l.eb + al((size_t)chunk * n * sizeof(int));
  l.total = l.err + al(sizeof(int));
  return l;
}

}  // namespace

extern "C" {

size_t khp_zgemm_fp64_tc_workspace(int64_t batch, int32_t m, int32_t n, int32_t k) {
  if (batch < 0 || m < 1 || n < 1 || k < 1) return 0;
  return abi_layout(ozaki_chunk(std::max<int64_t>(batch, 1)), m, n, k).total;
}

int khp_zgemm_fp64_tc(int64_t batch, int32_t m, int32_t n, int32_t k, const double* A, int64_t lda, int64_t bsA,
                      const double* B, int64_t ldb, int64_t bsB, double* C, int64_t ldc, int64_t bsC, void* workspace,
                      size_t ws_bytes, void* stream) {
  if (batch < 0 || m < 1 || n < 1 || k < 1 || k > 4096 || !A || !B || !C || lda < k || ldb < n || ldc < n)
    return KHP_ERR_INVALID_ARG;
  if (batch == 0) return KHP_OK;
  const int64_t chunk = ozaki_chunk(batch);
  const WsLayout l = abi_layout(chunk, m, n, k);
  if (!workspace || ws_bytes < l.total) return KHP_ERR_WORKSPACE;
  char* base = static_cast<char*>(workspace);
  OzakiWs w;
  w.ad = base + l.ad;
  w.ad_elems = (size_t)chunk * ozaki_a_elems(m, k);
  w.ea = reinterpret_cast<int*>(base + l.ea);
  w.ea_n = (size_t)chunk * ozaki_rows_padded(m);
  w.bd = base + l.bd;
  w.bd_elems = (size_t)chunk * ozaki_b_elems(k, n);
  w.eb = reinterpret_cast<int*>(base + l.eb);
  w.eb_n = (size_t)chunk * n;
  w.err = reinterpret_cast<int*>(base + l.err);
  return ozaki_zgemm(batch, m, n, k, reinterpret_cast<const cd*>(A), lda, bsA, nullptr,
                     reinterpret_cast<const cd*>(B), ldb, bsB, reinterpret_cast<cd*>(C), ldc, bsC, w,
                     reinterpret_cast<cudaStream_t>(stream));
}

}  // extern "C"
