// Exact digit products on the tcgen05 tensor cores, accumulated in tensor memory (TMEM).
//
// The operands are cut into ND signed 7-bit digits per row of A / column of B (integer bit
// arithmetic on the FP64 pattern: X = round(x 2^(7 ND - e)), digits from the low end in
// [-64, 63], the leading one |q_0| <= 128), so every digit is an exact bf16.  The complex product
// is the real product [Re A | Im A] [[Re B, Im B], [-Im B, Re B]] with the output columns
// interleaved (2c: Re C[:, c], 2c + 1: Im C[:, c]).  The digit pairs (i, j) with i + j = l < ND
// accumulate into level l's own TMEM accumulator (128 lanes x NT FP32 columns) over the whole
// inner dimension:
//   level 0:        K 2^14 per element,  level l >= 1:  K 2^12 (l + 3),
// so for K <= 576 the levels l <= 4 stay integers below 2^24, exact in FP32; the higher levels
// weigh 2^-35 and less and their rounding stays below 2^-59 of the result.  The epilogue
// combines the levels in 64-bit integers and converts once:
//   ND = 8 (FP64 result): sum_l L_l 2^-7(l+2) = hi 2^-35 + lo 2^-63 with hi, lo four levels each;
//   ND = 6 (FP64 result, 42-bit operands): the same with lo from levels 4 and 5;
//   ND = 4 (FP32 result): sum_l L_l 2^-7(l+2) = hi 2^-35, rounded once to FP32.
//
// Kernel: one CTA of 4 warps per 128 x NT tile of one problem's real output; one thread streams the
// digit tiles with TMA (cp.async.bulk.tensor, 128-byte swizzle), one thread issues tcgen05.mma
// (kind::f16, bf16 in, FP32 accumulate, M = 128, N = NT, K = 16) from shared-memory descriptors
// (K-major, 128-byte swizzle), full / empty mbarriers per buffer hand the tiles over, and all
// warps run the epilogue from TMEM (tcgen05.ld).  Every mbarrier wait is bounded: on time-out
// the CTA sets an error flag, frees TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "khepri_gb300.h"
#include "khp_core.cuh"
#include "khp_launch.h"

namespace khp {
namespace {

using bf16 = __nv_bfloat16;

constexpr int kM = 128;     // tile rows = TMEM lanes
constexpr int kK = 64;      // inner slice: one 128-byte row of bf16
constexpr uint32_t kTmemCols = 512;
constexpr int kThreads = 128;
constexpr long long kSpinLimit = 1ll << 26;  // mbarrier polls before giving up

template <int ND>
struct TcCfg;
template <>
struct TcCfg<8> {
  static constexpr int NT = 64;  // 8 levels x 64 columns = 512 TMEM columns
};
template <>
struct TcCfg<6> {
  static constexpr int NT = 64;  // 6 levels x 64 columns (of the 512 allocated)
};
template <>
struct TcCfg<4> {
  static constexpr int NT = 128;  // 4 levels x 128 columns
};

constexpr int kRing = 4;  // A digit tiles in flight (steps of lookahead + 1)

template <int ND>
constexpr size_t tc_smem_bytes() {
  return 1024 /* alignment slack */ + 2 * (size_t)ND * TcCfg<ND>::NT * 128 + kRing * (size_t)kM * 128;
}

inline int up_to(int x, int q) { return (x + q - 1) / q * q; }

// ---- digit splitting -------------------------------------------------------------------------
__device__ __forceinline__ int biased_exp(double x) {
  const uint64_t u = (uint64_t)__double_as_longlong(x);
  const int be = (int)((u >> 52) & 0x7ff);
  return be == 0 ? ((u << 1) != 0 ? 1 : 0) : be;
}
__device__ __forceinline__ int scale_exp(int bemax) { return bemax > 0 ? bemax - 1022 : 0; }

// ND signed 7-bit digits of x 2^-e (|x| < 2^e) into out[d * dstride]; NaN / inf give a NaN digit.
template <int ND>
__device__ __forceinline__ void put_digits7(double x, int e, bf16* out, int64_t dstride) {
  const uint64_t u = (uint64_t)__double_as_longlong(x);
  const int be = (int)((u >> 52) & 0x7ff);
  if (be == 0x7ff) {
    out[0] = __float2bfloat16_rn(__int_as_float(0x7fc00000));
#pragma unroll
    for (int d = 1; d < ND; ++d) out[d * dstride] = __float2bfloat16_rn(0.f);
    return;
  }
  const uint64_t frac = u & 0xfffffffffffffull;
  const uint64_t mant = be == 0 ? frac : (frac | (1ull << 52));
  const int sh = (be == 0 ? 1 : be) - 1075 + 7 * ND - e;  // X = mant 2^sh, |X| < 2^(7 ND)
  uint64_t mag;
  if (sh >= 0)
    mag = mant << sh;
  else if (sh > -63)
    mag = (mant + (1ull << (-sh - 1))) >> (-sh);
  else
    mag = 0;
  int64_t X = (u >> 63) ? -(int64_t)mag : (int64_t)mag;
#pragma unroll
  for (int d = ND - 1; d >= 1; --d) {
    const int q = (int)((X + 64) & 127) - 64;
    X = (X - q) >> 7;  // exact
    out[d * dstride] = __int2bfloat16_rn(q);
  }
  out[0] = __int2bfloat16_rn((int)X);
}

// A digits (rows of [Re A | Im A]), one warp per (problem, padded row); aidx optional.
template <int ND, typename TI>
__global__ void k_tc_split_a(int64_t batch, int m, int k, const cplx<TI>* __restrict__ A, int64_t lda, int64_t bsA,
                             const int* __restrict__ aidx, int Mp, int K2p, bf16* __restrict__ Ad,
                             int* __restrict__ ea) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; w < batch * Mp; w += nwarps) {
    const int64_t b = w / Mp;
    const int r = (int)(w % Mp);
    const bool live = r < m;
    const cplx<TI>* row = A + (aidx ? (int64_t)aidx[b] : b) * bsA + (int64_t)r * lda;
    int bm = 0;
    if (live)
      for (int kk = lane; kk < k; kk += 32)
        bm = max(bm, max(biased_exp((double)row[kk].re), biased_exp((double)row[kk].im)));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) bm = max(bm, __shfl_xor_sync(0xffffffffu, bm, o));
    const int ex = scale_exp(bm);
    if (lane == 0) ea[w] = ex;
    const int64_t ds = (int64_t)Mp * K2p;
    bf16* base = Ad + b * ND * ds + (int64_t)r * K2p;
    for (int kk = lane; kk < K2p; kk += 32) {
      double x = 0.0;
      if (live) x = kk < k ? (double)row[kk].re : (kk < 2 * k ? (double)row[kk - k].im : 0.0);
      put_digits7<ND>(x, ex, base + kk, ds);
    }
  }
}

// Column exponents of B, thread per (problem, column).
template <typename TI>
__global__ void k_tc_col_exp(int64_t batch, int k, int n, const cplx<TI>* __restrict__ B, int64_t ldb, int64_t bsB,
                             const int* __restrict__ bidx, int* __restrict__ eb) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < batch * n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / n;
    const int c = (int)(e % n);
    const cplx<TI>* col = B + (bidx ? (int64_t)bidx[b] : b) * bsB + c;
    int bm = 0;
    for (int kk = 0; kk < k; ++kk) {
      const cplx<TI> v = col[(int64_t)kk * ldb];
      bm = max(bm, max(biased_exp((double)v.re), biased_exp((double)v.im)));
    }
    eb[e] = scale_exp(bm);
  }
}

// B digits: real column j = 2 c + part, part 0: [Re B; -Im B] of column c, part 1: [Im B; Re B];
// zero outside 2n x 2k.  Block (32, 8): 32 real columns x 32 inner indices through shared memory
// (coalesced reads of B's rows, coalesced digit writes along the inner index).
template <int ND, typename TI>
__global__ void __launch_bounds__(256) k_tc_split_b(int k, int n, const cplx<TI>* __restrict__ B, int64_t ldb,
                                                    int64_t bsB, const int* __restrict__ bidx, int N2p, int K2p,
                                                    const int* __restrict__ eb, bf16* __restrict__ Bd) {
  __shared__ double xs[32][33];
  const int64_t b = blockIdx.z;
  const int j0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const cplx<TI>* Bb = B + (bidx ? (int64_t)bidx[b] : b) * bsB;
  {
    const int j = j0 + tx;
    const int c = j >> 1, part = j & 1;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int kl = ty + 8 * i;
      const int kk = k0 + kl;
      double x = 0.0;
      if (c < n && kk < 2 * k) {
        const cplx<TI> v = Bb[(int64_t)(kk < k ? kk : kk - k) * ldb + c];
        x = part == 0 ? (kk < k ? (double)v.re : -(double)v.im) : (kk < k ? (double)v.im : (double)v.re);
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
    const int ex = (j >> 1) < n ? eb[b * n + (j >> 1)] : 0;
    put_digits7<ND>(xs[tx][jl], ex, Bd + b * ND * per + (int64_t)j * K2p + k0 + tx, per);
  }
}

// ---- tcgen05 helpers -------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }


// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups 1024 bytes apart.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
  return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) | ((uint64_t)1 << 46) |
         ((uint64_t)2 << 61);
}

// Instruction descriptor of kind::f16: bf16 A and B (K-major), FP32 accumulator, M x N.
__host__ __device__ constexpr uint32_t instr_desc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accum) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum));
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar));
}

// Bounded wait for the phase of the given parity to complete; false on time-out.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
  uint32_t done = 0;
  for (long long it = 0; it < kSpinLimit && !done; ++it)
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(mbar), "r"(parity));
  return done != 0;
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

// ---- the product kernel ----------------------------------------------------------------------
// 2^e as a double built from its bits (normal range), else through ldexp.
__device__ __forceinline__ double pow2(int e) {
  return (e > -1023 && e < 1024) ? __longlong_as_double((long long)(e + 1023) << 52) : ldexp(1.0, e);
}
// (hi 2^-35 + lo 2^-63) 2^ex with two conversions, one product and one fused multiply-add
__device__ __forceinline__ double scaled_sum(long long hi, long long lo, int ex) {
  return fma((double)hi, pow2(ex - 35), (double)lo * pow2(ex - 63));
}
// hi 2^(ex - 35) rounded once to FP32
__device__ __forceinline__ float scaled_hi(long long hi, int ex) {
  const int e = ex - 35;
  const float h = (float)hi;
  return (e > -127 && e < 128) ? h * __int_as_float((e + 127) << 23) : ldexpf(h, e);
}

__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}
// TMA: box {64, rows, 1} of a 3-D digit tensor (inner index, row, digit plane) into shared memory,
// 128-byte swizzled; completion counted in bytes on mbar.
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* tmap, int x, int y, int z, uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
          dst),
      "l"(reinterpret_cast<uint64_t>(tmap)), "r"(x), "r"(y), "r"(z), "r"(mbar)
      : "memory");
}

// grid: (N2p / NT, Mp / 128, problems of this launch); C[b] (m x n complex) = alpha (A B) + beta C.
// Warp 0 lane 0 streams the digit tiles with TMA (A: one digit per step through a ring of kRing
// buffers; B: all ND digits of a 64-wide slice, double-buffered), warp 1 lane 0 issues the MMAs,
// and full / empty mbarriers per buffer hand the tiles over (empty ones are armed by
// tcgen05.commit when the MMAs reading a buffer have completed).  All four warps run the epilogue.
template <int ND, typename TO>
__global__ void __launch_bounds__(kThreads, 1)
    k_tc_digits(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int m, int n, int Mp,
                int K2p, const int* __restrict__ ea, const int* __restrict__ eb, cplx<TO>* C, int64_t ldc, int64_t bsC,
                cplx<TO> alpha, cplx<TO> beta, int use_beta, int* err) {
  constexpr int NT = TcCfg<ND>::NT;
  constexpr uint32_t kTileB = NT * 128;  // one digit's B tile (bytes)
  constexpr uint32_t kTileA = kM * 128;
  constexpr uint32_t kIdesc = instr_desc(kM, NT);
  extern __shared__ unsigned char dsm_raw[];
  __shared__ __align__(8) uint64_t afull[kRing], aempty[kRing], bfull[2], bempty[2], done;
  __shared__ uint32_t tmem_slot;
  __shared__ int s_err;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t base = (smem_u32(dsm_raw) + 1023u) & ~1023u;
  const uint32_t sB = base;                    // [2][ND][NT rows x 128 B]
  const uint32_t sA = base + 2 * ND * kTileB;  // [kRing][128 rows x 128 B]
  const int64_t b = blockIdx.z;
  const int S = K2p / kK;
  const int T = S * ND;
  const bool plain = !use_beta && alpha.re == TO(1) && alpha.im == TO(0);

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
#pragma unroll
    for (int q = 0; q < kRing; ++q) {
      mbar_init(smem_u32(&afull[q]), 1);
      mbar_init(smem_u32(&aempty[q]), 1);
    }
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      mbar_init(smem_u32(&bfull[q]), 1);
      mbar_init(smem_u32(&bempty[q]), 1);
    }
    mbar_init(smem_u32(&done), 1);
    asm volatile("fence.mbarrier_init.release.cluster;");
    s_err = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_slot;

  if (warp == 0 && lane == 0) {
    // producer: the u-th refill of a buffer waits for the (u-1)-th release (parity (u & 1) ^ 1:
    // the phase before the first is complete)
    for (int t = 0; t < T && !s_err; ++t) {
      const int s = t / ND, i = t % ND;
      if (i == 0) {
        const int bs = s & 1;
        if (!mbar_wait(smem_u32(&bempty[bs]), (uint32_t)(((s >> 1) & 1) ^ 1))) {
          atomicExch(&s_err, 1);
          break;
        }
        mbar_expect_tx(smem_u32(&bfull[bs]), (uint32_t)ND * kTileB);
#pragma unroll
        for (int d = 0; d < ND; ++d)
          tma_load_3d(sB + (bs * ND + d) * kTileB, &tmB, s * kK, blockIdx.x * NT, (int)b * ND + d,
                      smem_u32(&bfull[bs]));
      }
      const int as = t % kRing;
      if (!mbar_wait(smem_u32(&aempty[as]), (uint32_t)(((t / kRing) & 1) ^ 1))) {
        atomicExch(&s_err, 1);
        break;
      }
      mbar_expect_tx(smem_u32(&afull[as]), kTileA);
      tma_load_3d(sA + as * kTileA, &tmA, s * kK, blockIdx.y * kM, (int)b * ND + i, smem_u32(&afull[as]));
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    for (int t = 0; t < T && !s_err; ++t) {
      const int s = t / ND, i = t % ND, as = t % kRing;
      if (i == 0 && !mbar_wait(smem_u32(&bfull[s & 1]), (uint32_t)((s >> 1) & 1))) {
        atomicExch(&s_err, 1);
        break;
      }
      if (!mbar_wait(smem_u32(&afull[as]), (uint32_t)((t / kRing) & 1))) {
        atomicExch(&s_err, 1);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      // descriptors differ only in their start-address field: one base each, then 16-byte units
      const uint64_t adesc = smem_desc(sA + as * kTileA);
      const uint64_t bdesc = smem_desc(sB + (s & 1) * ND * kTileB);
      const uint32_t acc0 = t == 0 ? 0u : 1u;
#pragma unroll
      for (int j = 0; j < ND; ++j) {
        if (j + i >= ND) break;
        const uint32_t d = tmem + (uint32_t)((i + j) * NT);
        const uint64_t bj = bdesc + (uint64_t)(j * (kTileB >> 4));
        mma_bf16(d, adesc, bj, kIdesc, acc0);
        mma_bf16(d, adesc + 2, bj + 2, kIdesc, 1u);
        mma_bf16(d, adesc + 4, bj + 4, kIdesc, 1u);
        mma_bf16(d, adesc + 6, bj + 6, kIdesc, 1u);
      }
      mma_commit(smem_u32(&aempty[as]));
      if (i == ND - 1) mma_commit(smem_u32(&bempty[s & 1]));
    }
    mma_commit(smem_u32(&done));
  }
  __syncwarp();
  const bool finished = mbar_wait(smem_u32(&done), 0u);
  if (!finished) atomicExch(&s_err, 1);
  __syncthreads();
  if (!s_err) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    const int r = blockIdx.y * kM + tid;  // lane (32 warp + lane) = tile row
    const int ex_a = r < m ? ea[b * Mp + r] : 0;
    cplx<TO>* Cb = C + b * bsC;
    for (int cc = 0; cc < NT; cc += 16) {
      uint32_t v[ND][16];
#pragma unroll
      for (int l = 0; l < ND; ++l) tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(l * NT + cc), v[l]);
      asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
      for (int q = 0; q < 16; q += 2) {
        const int col = blockIdx.x * NT + cc + q;  // interleaved: col = 2 c (Re), 2 c + 1 (Im)
        const int c = col >> 1;
        if (r >= m || c >= n) continue;
        const int ex = ex_a + eb[b * n + c];
        TO out[2];
#pragma unroll
        for (int p = 0; p < 2; ++p) {
          // level sums are integers below 2^31: 32-bit conversions, 64-bit integer combination
          long long hi = 0;
#pragma unroll
          for (int l = 0; l < 4; ++l)
            hi += (long long)__float2int_rn(__uint_as_float(v[l][q + p])) * (1ll << (7 * (3 - l)));
          if constexpr (ND > 4) {
            long long lo = 0;
#pragma unroll
            for (int l = 4; l < ND; ++l)
              lo += (long long)__float2int_rn(__uint_as_float(v[l][q + p])) * (1ll << (7 * (7 - l)));
            out[p] = (TO)scaled_sum(hi, lo, ex);
          } else {
            out[p] = (TO)scaled_hi(hi, ex);
          }
        }
        cplx<TO>* dst = Cb + (int64_t)r * ldc + c;
        if (plain) {
          *dst = mk(out[0], out[1]);
        } else {
          cplx<TO> val = alpha * mk(out[0], out[1]);
          if (use_beta) val += beta * *dst;
          *dst = val;
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
  if (tid == 0 && s_err) atomicExch(err, 1);
}

// A CTA that timed out waiting for its products leaves its tile unwritten: mark every problem's
// result non-finite so that the callers' status words report it.
template <typename TO>
__global__ void k_tc_poison(const int* err, int64_t batch, cplx<TO>* C, int64_t bsC) {
  if (*err == 0) return;
  for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < batch; b += (int64_t)gridDim.x * blockDim.x)
    C[b * bsC] = mk(TO(NAN), TO(NAN));
}

// cuTensorMapEncodeTiled from the driver (looked up once through the runtime).
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
}

// 3-D bf16 digit tensor [planes][rows][K2p] with 64 x box_rows boxes, 128-byte swizzle.
bool encode_digits_map(CUtensorMap* map, const bf16* base, int K2p, int rows, int64_t planes, int box_rows) {
  const EncodeTiledFn fn = encode_fn();
  if (!fn) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)K2p, (cuuint64_t)rows, (cuuint64_t)planes};
  const cuuint64_t strides[2] = {(cuuint64_t)K2p * 2, (cuuint64_t)rows * K2p * 2};
  const cuuint32_t box[3] = {(cuuint32_t)kK, (cuuint32_t)box_rows, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<bf16*>(base), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

inline unsigned grid_of(int64_t total, int threads) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((total + threads - 1) / threads, 152 * 32));
}

// ---- 3xTF32 products -------------------------------------------------------------------------
// C = alpha A B + beta C for complex FP32 A (m x k) and B (k x n), as one real product over the
// inner index i = 2t + q (q = 0: Re, 1: Im): row r of A' is A's own interleaved row r; row
// j = 2c + p of B' (one real output column, p = 0: Re C[:, c], 1: Im) holds, at i = 2t + q, entry
// (p, q) of [[Re b, -Im b], [Im b, Re b]] for b = B[t][c].  Every operand value is split
// x = hi + lo with hi = x rounded to TF32 and lo = x - hi (exact in FP32) rounded to TF32, and the
// tile accumulates hi hi' + hi lo' + lo hi' in one FP32 TMEM accumulator; the dropped lo lo' term
// is ~2^-22 of the product and the rounding of lo ~2^-21: FP32 accuracy at the TF32 tensor rate.
// Operand planes: [problems][2 (hi, lo)][rows padded to 128][inner padded to 32] FP32.

constexpr int kTfNT = 128;    // real output columns per tile
constexpr int kTfK = 32;      // inner slice: one 128-byte row of FP32
constexpr int kTfStages = 3;  // slices in flight (3 x 64 KB of shared memory)
constexpr uint32_t kTfTmemCols = 128;

inline int tf_rows(int r) { return up_to(r, kM); }
inline int tf_inner(int k) { return up_to(2 * k, kTfK); }
constexpr size_t tf_smem_bytes() { return 1024 + (size_t)kTfStages * 4 * kM * 128; }

__device__ __forceinline__ void tf32_split(float x, float& hi, float& lo) {
  uint32_t h, l;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(x));
  hi = __uint_as_float(h);
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(l) : "f"(x - hi));
  lo = __uint_as_float(l);
}

// A' planes: a block per (problem, padded row) at a time, threads along the inner index (A's row
// read as consecutive floats, re and im interleaved exactly as i = 2t + q); aidx optional.
__global__ void __launch_bounds__(256) k_tf_split_a(int64_t batch, int m, int k, const cplx<float>* __restrict__ A,
                                                    int64_t lda, int64_t bsA, const int* __restrict__ aidx, int Mp,
                                                    int Kp, float* __restrict__ out) {
  const int64_t per = (int64_t)Mp * Kp;
  for (int64_t row = blockIdx.x; row < batch * Mp; row += gridDim.x) {
    const int64_t b = row / Mp;
    const int r = (int)(row - b * Mp);
    const float* src = reinterpret_cast<const float*>(A + (aidx ? (int64_t)aidx[b] : b) * bsA + (int64_t)r * lda);
    float* hi_p = out + b * 2 * per + (int64_t)r * Kp;
    for (int i = threadIdx.x; i < Kp; i += blockDim.x) {
      const float x = (r < m && i < 2 * k) ? src[i] : 0.f;
      float hi, lo;
      tf32_split(x, hi, lo);
      hi_p[i] = hi;
      hi_p[per + i] = lo;
    }
  }
}

// B' planes of B + shift I through shared memory: a block (32, 8) reads a 16 x 16 tile of B (rows
// t, columns c; coalesced along c) and writes the 32 x 32 tile of B' (rows j = 2c + p, inner
// i = 2t + q; coalesced along i).
__global__ void __launch_bounds__(256) k_tf_split_b(int k, int n, const cplx<float>* __restrict__ B, int64_t ldb,
                                                    int64_t bsB, const int* __restrict__ bidx, int Np, int Kp,
                                                    cplx<float> shift, float* __restrict__ out) {
  __shared__ cplx<float> tile[16][17];
  const int64_t b = blockIdx.z;
  const int c0 = blockIdx.x * 16, t0 = blockIdx.y * 16;
  const int tid = threadIdx.y * 32 + threadIdx.x;
  const cplx<float>* Bb = B + (bidx ? (int64_t)bidx[b] : b) * bsB;
  {
    const int tl = tid >> 4, cl = tid & 15;
    const int t = t0 + tl, c = c0 + cl;
    cplx<float> v = (t < k && c < n) ? Bb[(int64_t)t * ldb + c] : mk(0.f);
    if (t == c && t < k && c < n) v += shift;  // B + shift I
    tile[tl][cl] = v;
  }
  __syncthreads();
  const int64_t per = (int64_t)Np * Kp;
  float* hi_p = out + b * 2 * per;
  float* lo_p = hi_p + per;
  const int il = threadIdx.x;  // inner index in the tile: t = il >> 1, q = il & 1
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int jl = threadIdx.y + 8 * u;  // output row in the tile: c = jl >> 1, p = jl & 1
    const cplx<float> v = tile[il >> 1][jl >> 1];
    const int p = jl & 1, q = il & 1;
    const float x = p == 0 ? (q == 0 ? v.re : -v.im) : (q == 0 ? v.im : v.re);
    float hi, lo;
    tf32_split(x, hi, lo);
    const int64_t o = (int64_t)(2 * c0 + jl) * Kp + 2 * t0 + il;
    hi_p[o] = hi;
    lo_p[o] = lo;
  }
}

// Instruction descriptor of kind::tf32: TF32 A and B (K-major), FP32 accumulator, M x N.
__host__ __device__ constexpr uint32_t instr_desc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accum) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum));
}

// grid: (Np / 128, Mp / 128, problems of this launch).  Warp 0 lane 0 loads each 32-wide inner
// slice's four tiles (A hi, A lo, B hi, B lo) with TMA into a ring of kTfStages buffers, warp 1
// lane 0 issues the 3 x 4 MMAs of the slice (K = 8 each) and releases the buffer through its
// empty mbarrier, and all four warps run the epilogue from TMEM.  Every wait is bounded: on
// time-out the CTA sets the error flag, frees TMEM and returns.
__global__ void __launch_bounds__(kThreads, 1)
    k_tf32x3(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int m, int n, int Kp,
             cplx<float>* C, int64_t ldc, int64_t bsC, cplx<float> alpha, cplx<float> beta, int use_beta, int* err) {
  constexpr uint32_t kTile = kM * 128;  // 128 rows x 32 FP32 (A and B tiles alike, kTfNT == kM)
  constexpr uint32_t kStage = 4 * kTile;
  constexpr uint32_t kIdesc = instr_desc_tf32(kM, kTfNT);
  extern __shared__ unsigned char dsm_raw[];
  __shared__ __align__(8) uint64_t full[kTfStages], empty[kTfStages], done;
  __shared__ uint32_t tmem_slot;
  __shared__ int s_err;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t base = (smem_u32(dsm_raw) + 1023u) & ~1023u;
  const int64_t b = blockIdx.z;
  const int S = Kp / kTfK;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(kTfTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
#pragma unroll
    for (int q = 0; q < kTfStages; ++q) {
      mbar_init(smem_u32(&full[q]), 1);
      mbar_init(smem_u32(&empty[q]), 1);
    }
    mbar_init(smem_u32(&done), 1);
    asm volatile("fence.mbarrier_init.release.cluster;");
    s_err = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_slot;

  if (warp == 0 && lane == 0) {
    for (int sl = 0; sl < S && !s_err; ++sl) {
      const int st = sl % kTfStages;
      if (!mbar_wait(smem_u32(&empty[st]), (uint32_t)(((sl / kTfStages) & 1) ^ 1))) {
        atomicExch(&s_err, 1);
        break;
      }
      const uint32_t buf = base + st * kStage;
      mbar_expect_tx(smem_u32(&full[st]), kStage);
      tma_load_3d(buf, &tmA, sl * kTfK, blockIdx.y * kM, (int)b * 2, smem_u32(&full[st]));
      tma_load_3d(buf + kTile, &tmA, sl * kTfK, blockIdx.y * kM, (int)b * 2 + 1, smem_u32(&full[st]));
      tma_load_3d(buf + 2 * kTile, &tmB, sl * kTfK, blockIdx.x * kTfNT, (int)b * 2, smem_u32(&full[st]));
      tma_load_3d(buf + 3 * kTile, &tmB, sl * kTfK, blockIdx.x * kTfNT, (int)b * 2 + 1, smem_u32(&full[st]));
    }
  } else if (warp == 1 && lane == 0) {
    for (int sl = 0; sl < S && !s_err; ++sl) {
      const int st = sl % kTfStages;
      if (!mbar_wait(smem_u32(&full[st]), (uint32_t)((sl / kTfStages) & 1))) {
        atomicExch(&s_err, 1);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t buf = base + st * kStage;
      const uint64_t ahi = smem_desc(buf), alo = smem_desc(buf + kTile);
      const uint64_t bhi = smem_desc(buf + 2 * kTile), blo = smem_desc(buf + 3 * kTile);
#pragma unroll
      for (int kk = 0; kk < kTfK / 8; ++kk) {
        const uint64_t o = (uint64_t)(2 * kk);  // 32 bytes per K = 8 step, in 16-byte units
        mma_tf32(tmem, ahi + o, bhi + o, kIdesc, (sl == 0 && kk == 0) ? 0u : 1u);
        mma_tf32(tmem, ahi + o, blo + o, kIdesc, 1u);
        mma_tf32(tmem, alo + o, bhi + o, kIdesc, 1u);
      }
      mma_commit(smem_u32(&empty[st]));
    }
    mma_commit(smem_u32(&done));
  }
  __syncwarp();
  const bool finished = mbar_wait(smem_u32(&done), 0u);
  if (!finished) atomicExch(&s_err, 1);
  __syncthreads();
  if (!s_err) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    const int r = blockIdx.y * kM + tid;  // TMEM lane (32 warp + lane) = tile row
    cplx<float>* Cb = C + b * bsC;
    const bool plain = !use_beta && alpha.re == 1.f && alpha.im == 0.f;
    for (int cc = 0; cc < kTfNT; cc += 16) {
      uint32_t v[16];
      tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)cc, v);
      asm volatile("tcgen05.wait::ld.sync.aligned;");
      if (r >= m) continue;
#pragma unroll
      for (int q = 0; q < 16; q += 2) {
        const int c = (blockIdx.x * kTfNT + cc + q) >> 1;
        if (c >= n) continue;
        const cplx<float> val = mk(__uint_as_float(v[q]), __uint_as_float(v[q + 1]));
        cplx<float>* dst = Cb + (int64_t)r * ldc + c;
        if (plain) {
          *dst = val;
        } else {
          cplx<float> o = alpha * val;
          if (use_beta) o += beta * *dst;
          *dst = o;
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTfTmemCols));
  if (tid == 0 && s_err) atomicExch(err, 1);
}

// 3-D FP32 operand planes [planes][rows][Kp] with 32 x 128 boxes, 128-byte swizzle.
bool encode_planes_map(CUtensorMap* map, const float* base, int Kp, int rows, int64_t planes) {
  const EncodeTiledFn fn = encode_fn();
  if (!fn) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)Kp, (cuuint64_t)rows, (cuuint64_t)planes};
  const cuuint64_t strides[2] = {(cuuint64_t)Kp * 4, (cuuint64_t)rows * Kp * 4};
  const cuuint32_t box[3] = {(cuuint32_t)kTfK, (cuuint32_t)kM, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

// Largest inner size (2k padded to 64) for which the levels that matter stay exact.
int tc_max_k2p(int nd) { return nd > 4 ? 576 : 640; }

size_t tc_a_elems(int nd, int m, int k) { return (size_t)nd * up_to(m, kM) * up_to(2 * k, kK); }
size_t tc_b_elems(int nd, int k, int n) {
  const int nt = nd > 4 ? TcCfg<8>::NT : TcCfg<4>::NT;
  return (size_t)nd * up_to(2 * n, nt) * up_to(2 * k, kK);
}
int tc_rows_padded(int m) { return up_to(m, kM); }

template <int ND, typename TI, typename TO>
int tc_product(int64_t batch, int m, int n, int k, const cplx<TI>* A, int64_t lda, int64_t bsA, const int* aidx,
               const cplx<TI>* B, int64_t ldb, int64_t bsB, const int* bidx, cplx<TO> alpha, cplx<TO> beta,
               cplx<TO>* C, int64_t ldc, int64_t bsC, const OzakiWs& w, cudaStream_t s) {
  constexpr int NT = TcCfg<ND>::NT;
  const int Mp = up_to(m, kM), N2p = up_to(2 * n, NT), K2p = up_to(2 * k, kK);
  if (K2p > tc_max_k2p(ND)) return KHP_ERR_INVALID_ARG;
  const int64_t per_a = (int64_t)ND * Mp * K2p, per_b = (int64_t)ND * N2p * K2p;
  const int64_t chunk = std::min(std::min<int64_t>((int64_t)(w.ad_elems / per_a), (int64_t)(w.ea_n / Mp)),
                                 std::min<int64_t>((int64_t)(w.bd_elems / per_b), (int64_t)(w.eb_n / n)));
  if (chunk <= 0) return KHP_ERR_WORKSPACE;
  const size_t smem = tc_smem_bytes<ND>();
  if (cudaFuncSetAttribute(k_tc_digits<ND, TO>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return KHP_ERR_CUDA;
  const bool use_beta = !(beta.re == TO(0) && beta.im == TO(0));
  if (!w.err) return KHP_ERR_WORKSPACE;
  if (cudaMemsetAsync(w.err, 0, sizeof(int), s) != cudaSuccess) return KHP_ERR_CUDA;
  stage_begin(KHP_STAGE_TC_PRODUCT, s);
  for (int64_t off = 0; off < batch; off += chunk) {
    const int64_t nb = std::min<int64_t>(chunk, batch - off);
    bf16* Adg = static_cast<bf16*>(w.ad);
    bf16* Bdg = static_cast<bf16*>(w.bd);
    k_tc_split_a<ND, TI><<<grid_of(nb * Mp * 32, 256), 256, 0, s>>>(
        nb, m, k, aidx ? A : A + off * bsA, lda, bsA, aidx ? aidx + off : nullptr, Mp, K2p, Adg, w.ea);
    k_tc_col_exp<TI><<<grid_of(nb * n, 128), 128, 0, s>>>(nb, k, n, bidx ? B : B + off * bsB, ldb, bsB,
                                                         bidx ? bidx + off : nullptr, w.eb);
    count_launches(2);
    for (int64_t o2 = 0; o2 < nb; o2 += 65535) {
      const unsigned z = (unsigned)std::min<int64_t>(nb - o2, 65535);
      const int64_t bo = off + o2;
      k_tc_split_b<ND, TI><<<dim3(N2p / 32, K2p / 32, z), dim3(32, 8), 0, s>>>(
          k, n, bidx ? B : B + bo * bsB, ldb, bsB, bidx ? bidx + bo : nullptr, N2p, K2p, w.eb + o2 * n,
          Bdg + o2 * per_b);
      CUtensorMap tmA, tmB;
      if (!encode_digits_map(&tmA, Adg + o2 * per_a, K2p, Mp, (int64_t)z * ND, kM) ||
          !encode_digits_map(&tmB, Bdg + o2 * per_b, K2p, N2p, (int64_t)z * ND, NT))
        return KHP_ERR_CUDA;
      k_tc_digits<ND, TO><<<dim3(N2p / NT, Mp / kM, z), kThreads, smem, s>>>(
          tmA, tmB, m, n, Mp, K2p, w.ea + o2 * Mp, w.eb + o2 * n, C + bo * bsC, ldc, bsC, alpha, beta,
          use_beta ? 1 : 0, w.err);
      count_launches(2);
    }
    const int st = cuda_status();
    if (st) return st;
  }
  k_tc_poison<TO><<<grid_of(batch, 128), 128, 0, s>>>(w.err, batch, C, bsC);
  count_launches(1);
  stage_end(KHP_STAGE_TC_PRODUCT, s);
  return cuda_status();
}

size_t tf32x3_a_elems(int m, int k) { return 2 * (size_t)tf_rows(m) * tf_inner(k); }
size_t tf32x3_b_elems(int k, int n) { return 2 * (size_t)up_to(2 * n, kTfNT) * tf_inner(k); }

int tf32x3_split_a(int64_t batch, int m, int k, const cplx<float>* A, int64_t lda, int64_t bsA, const int* aidx,
                   float* planes, cudaStream_t s) {
  const int Mp = tf_rows(m), Kp = tf_inner(k);
  const unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>(batch * Mp, 152 * 16));
  k_tf_split_a<<<blocks, 256, 0, s>>>(batch, m, k, A, lda, bsA, aidx, Mp, Kp, planes);
  count_launches(1);
  return cuda_status();
}

int tf32x3_split_b(int64_t batch, int k, int n, const cplx<float>* B, int64_t ldb, int64_t bsB, const int* bidx,
                   cplx<float> shift, float* planes, cudaStream_t s) {
  const int Np = up_to(2 * n, kTfNT), Kp = tf_inner(k);
  const int64_t per = (int64_t)2 * Np * Kp;
  for (int64_t off = 0; off < batch; off += 65535) {
    const unsigned z = (unsigned)std::min<int64_t>(batch - off, 65535);
    k_tf_split_b<<<dim3((unsigned)(Np / 32), (unsigned)(Kp / 32), z), dim3(32, 8), 0, s>>>(
        k, n, bidx ? B : B + off * bsB, ldb, bsB, bidx ? bidx + off : nullptr, Np, Kp, shift, planes + off * per);
    count_launches(1);
  }
  return cuda_status();
}

int tf32x3_from_planes(int64_t batch, int m, int n, int k, const float* Aplanes, const float* Bplanes,
                       cplx<float> alpha, cplx<float> beta, cplx<float>* C, int64_t ldc, int64_t bsC, int* err,
                       cudaStream_t s) {
  const int Mp = tf_rows(m), Np = up_to(2 * n, kTfNT), Kp = tf_inner(k);
  if (m < 1 || n < 1 || k < 1) return KHP_ERR_INVALID_ARG;
  const size_t smem = tf_smem_bytes();
  if (cudaFuncSetAttribute(k_tf32x3, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return KHP_ERR_CUDA;
  if (!err) return KHP_ERR_WORKSPACE;
  const bool use_beta = !(beta.re == 0.f && beta.im == 0.f);
  if (cudaMemsetAsync(err, 0, sizeof(int), s) != cudaSuccess) return KHP_ERR_CUDA;
  const int64_t per_a = 2 * (int64_t)Mp * Kp, per_b = 2 * (int64_t)Np * Kp;
  for (int64_t off = 0; off < batch; off += 65535) {
    const unsigned z = (unsigned)std::min<int64_t>(batch - off, 65535);
    CUtensorMap tmA, tmB;
    if (!encode_planes_map(&tmA, Aplanes + off * per_a, Kp, Mp, 2 * (int64_t)z) ||
        !encode_planes_map(&tmB, Bplanes + off * per_b, Kp, Np, 2 * (int64_t)z))
      return KHP_ERR_CUDA;
    k_tf32x3<<<dim3(Np / kTfNT, Mp / kM, z), kThreads, smem, s>>>(tmA, tmB, m, n, Kp, C + off * bsC, ldc, bsC, alpha,
                                                                   beta, use_beta ? 1 : 0, err);
    count_launches(1);
  }
  k_tc_poison<float><<<grid_of(batch, 128), 128, 0, s>>>(err, batch, C, bsC);
  count_launches(1);
  return cuda_status();
}

template int tc_product<8, double, double>(int64_t, int, int, int, const cplx<double>*, int64_t, int64_t, const int*,
                                           const cplx<double>*, int64_t, int64_t, const int*, cplx<double>,
                                           cplx<double>, cplx<double>*, int64_t, int64_t, const OzakiWs&,
                                           cudaStream_t);
template int tc_product<6, double, double>(int64_t, int, int, int, const cplx<double>*, int64_t, int64_t, const int*,
                                           const cplx<double>*, int64_t, int64_t, const int*, cplx<double>,
                                           cplx<double>, cplx<double>*, int64_t, int64_t, const OzakiWs&,
                                           cudaStream_t);
template int tc_product<4, float, float>(int64_t, int, int, int, const cplx<float>*, int64_t, int64_t, const int*,
                                         const cplx<float>*, int64_t, int64_t, const int*, cplx<float>, cplx<float>,
                                         cplx<float>*, int64_t, int64_t, const OzakiWs&, cudaStream_t);

}  // namespace khp

extern "C" {

size_t khp_cgemm_tf32x3_workspace(int64_t batch, int32_t m, int32_t n, int32_t k) {
  if (batch < 0 || m < 1 || n < 1 || k < 1) return 0;
  const size_t a = (sizeof(float) * khp::tf32x3_a_elems(m, k) * (size_t)batch + 255) & ~size_t(255);
  const size_t b = (sizeof(float) * khp::tf32x3_b_elems(k, n) * (size_t)batch + 255) & ~size_t(255);
  return a + b + 256;
}

int khp_cgemm_tf32x3(int64_t batch, int32_t m, int32_t n, int32_t k, const float* A, int64_t lda, int64_t a_stride,
                     const float* B, int64_t ldb, int64_t b_stride, float* C, int64_t ldc, int64_t c_stride,
                     void* workspace, size_t ws_bytes, void* stream) {
  using namespace khp;
  if (batch < 0 || m < 1 || n < 1 || k < 1 || !A || !B || !C || lda < k || ldb < n || ldc < n || a_stride < 0 ||
      b_stride < 0 || c_stride < 0)
    return KHP_ERR_INVALID_ARG;
  if (batch == 0) return KHP_OK;
  if (!workspace || ws_bytes < khp_cgemm_tf32x3_workspace(batch, m, n, k)) return KHP_ERR_WORKSPACE;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  char* w = static_cast<char*>(workspace);
  float* ap = reinterpret_cast<float*>(w);
  const size_t a = (sizeof(float) * tf32x3_a_elems(m, k) * (size_t)batch + 255) & ~size_t(255);
  float* bp = reinterpret_cast<float*>(w + a);
  const size_t b = (sizeof(float) * tf32x3_b_elems(k, n) * (size_t)batch + 255) & ~size_t(255);
  int* err = reinterpret_cast<int*>(w + a + b);
  const auto* Ac = reinterpret_cast<const cplx<float>*>(A);
  const auto* Bc = reinterpret_cast<const cplx<float>*>(B);
  auto* Cc = reinterpret_cast<cplx<float>*>(C);
  int st = tf32x3_split_a(batch, m, k, Ac, lda, a_stride, nullptr, ap, s);
  if (!st) st = tf32x3_split_b(batch, k, n, Bc, ldb, b_stride, nullptr, mk(0.f), bp, s);
  if (!st) st = tf32x3_from_planes(batch, m, n, k, ap, bp, mk(1.f), mk(0.f), Cc, ldc, c_stride, err, s);
  return st;
}

}  // extern "C"
