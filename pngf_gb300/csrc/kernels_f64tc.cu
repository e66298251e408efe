// FP64-accurate rank-k update of M on the tcgen05 tensor cores.
//
// GB300 runs FP64 at ~1.1 TFLOP/s, so the FP64 accept update M -= A W
// (8k(N+E)(N+1) flops) is FP64-pipe bound on the SIMT units. This path
// computes the same product with exact integer arithmetic on the BF16 tensor
// cores (the splitting method of Ozaki et al., "Error-free transformations of
// matrix multiplication by using fast routines of matrix multiplication and
// its applications", Numer. Algorithms 59, 2012):
//
//  * real form as in the complex64 path: A_real (rows x 2k, interleaved re/im)
//    and B_real (2(N+1) output columns x 2k);
//  * every row of A_real is scaled by a power of two 2^-e so that its largest
//    entry is below 1, then cut into 7 slices of 7 bits: x = sum_p a_p 2^-7p +
//    r, |r| < 2^-49, with integer a_p (|a_1| <= 128, |a_p| <= 64), exact in
//    BF16; likewise every row of B_real with 2^-f;
//  * products of slice pairs are exact in the tensor core and their sums over
//    K stay integers below 2^24 (k <= 128), so the FP32 accumulation in TMEM is
//    exact. Pairs with p + q = l share one accumulator per level l = 2..8 (28
//    pairs in 7 TMEM accumulators); pairs with p + q > 8 are dropped, an error
//    below 2^-50 of the row/column scales -- finer than FP64 GEMM rounding;
//  * the epilogue recombines the levels exactly in 64-bit integers,
//    Y = sum_l C_l 2^(7(7-l)), converts once and applies M -= Y 2^(e+f-49)
//    with one FP64 fused multiply-add per element.
//
// Kernel k_tc_update_f64: one CTA per 128-row x 64-column tile of M (as
// doubles), the whole K extent of both operands in shared memory (TMA,
// 128B swizzle), 28 pairs x 2k/16 tcgen05.mma.kind::f16 (M=128, N=64, K=16)
// issued by one thread into a 512-column TMEM allocation, 4 epilogue warps.
// Waits are bounded as in the complex64 kernel.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cstdint>
#include <mutex>

#include "pngf_internal.h"
#include "tc_common.cuh"

namespace pngf {

namespace {

using namespace tc;

constexpr int FB_BM = 128;   // rows of M per tile
constexpr int FB_BN = 64;    // double columns of M per tile (MMA N)
constexpr int FB_S = 7;      // slices per operand
constexpr int FB_B = 7;      // bits per slice
constexpr int FB_LMAX = 8;   // highest level kept (p + q <= 8)
constexpr int FB_NLEV = FB_LMAX - 1;  // levels 2..8
constexpr uint32_t FB_ATOM_A = FB_BM * 128;  // one 64-element K atom of the A tile
constexpr uint32_t FB_ATOM_B = FB_BN * 128;
constexpr int FB_MAX_ATOMS = 7;             // K extent up to 448 (k <= 32)
constexpr size_t FB_SMEM = FB_MAX_ATOMS * (FB_ATOM_A + FB_ATOM_B) + 1024 + 512;

// kind::f16 instruction descriptor: D f32, A and B bf16, K-major, N = 64, M = 128.
constexpr uint32_t kIdescBF16 =
    (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(FB_BN >> 3) << 17) | ((uint32_t)(FB_BM >> 4) << 24);

__device__ __forceinline__ int scale_exp(double m) {
  if (m == 0.0) return 0;
  return ilogb(m) + 1;  // m * 2^-e < 1
}

// Writes the 7 slices of x * 2^-e (|x 2^-e| < 1) into dst[0], dst[stride], ...
__device__ __forceinline__ void write_slices(double x, int e, __nv_bfloat16 *dst, int stride) {
  double r = ldexp(x, -e);
#pragma unroll
  for (int p = 0; p < FB_S; ++p) {
    const double t = r * 128.0;
    const double a = rint(t);
    r = t - a;
    dst[p * stride] = __float2bfloat16_rn((float)a);
  }
}

// A_op row i (i < rows): slices of the interleaved real row of A[i, :].
// Row layout: slice p at columns [p*k2p, p*k2p + 2k), zeros elsewhere up to kop.
__global__ void k_slice_A(const double2 *__restrict__ A, long lda, long rows, int k, int k2p, int kop,
                          __nv_bfloat16 *__restrict__ Aop, int *__restrict__ eA) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows) return;
  double m = 0.0;
  for (int r = 0; r < k; ++r) {
    const double2 a = A[(size_t)r * lda + i];
    m = fmax(m, fmax(fabs(a.x), fabs(a.y)));
  }
  const int e = scale_exp(m);
  eA[i] = e;
  __nv_bfloat16 *row = Aop + (size_t)i * kop;
  for (int c = 0; c < kop; ++c) row[c] = __float2bfloat16_rn(0.f);
  for (int r = 0; r < k; ++r) {
    const double2 a = A[(size_t)r * lda + i];
    write_slices(a.x, e, row + 2 * r, k2p);
    write_slices(a.y, e, row + 2 * r + 1, k2p);
  }
}

// B_op row j' < 2(N+1): output column j' = 2j (real part) or 2j+1 (imaginary)
// of M[:, j]; W is k x ldw (row-major, complex).
__global__ void k_slice_B(const double2 *__restrict__ W, long ldw, long ncols2, int k, int k2p, int kop,
                          __nv_bfloat16 *__restrict__ Bop, int *__restrict__ fB) {
  const long jp = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (jp >= ncols2) return;
  const long j = jp >> 1;
  const bool im = jp & 1;
  double m = 0.0;
  for (int r = 0; r < k; ++r) {
    const double2 w = W[(size_t)r * ldw + j];
    m = fmax(m, fmax(fabs(w.x), fabs(w.y)));
  }
  const int f = scale_exp(m);
  fB[jp] = f;
  __nv_bfloat16 *row = Bop + (size_t)jp * kop;
  for (int c = 0; c < kop; ++c) row[c] = __float2bfloat16_rn(0.f);
  for (int r = 0; r < k; ++r) {
    const double2 w = W[(size_t)r * ldw + j];
    // Re out: Re A Re W - Im A Im W; Im out: Re A Im W + Im A Re W
    write_slices(im ? w.y : w.x, f, row + 2 * r, k2p);
    write_slices(im ? w.x : -w.y, f, row + 2 * r + 1, k2p);
  }
}

// Exact int32 value of a float holding an integer of magnitude below 2^22:
// adding 1.5 * 2^23 puts the integer in the low mantissa bits (FP32 pipe only).
__device__ __forceinline__ int f2i_exact(float v) { return __float_as_int(v + 12582912.0f) - 0x4B400000; }

// Y * 2^E as a double, built from the bits on the integer pipe (round half
// up to 53 bits). Falls back to ldexp outside the normal exponent range.
__device__ __forceinline__ double i64_scaled(long long Y, int E) {
  if (Y == 0) return 0.0;
  const unsigned long long s = Y < 0 ? 1ull : 0ull;
  unsigned long long u = Y < 0 ? (unsigned long long)(-Y) : (unsigned long long)Y;
  int msb = 63 - __clzll((long long)u);
  unsigned long long mant;
  if (msb > 52) {
    const int sh = msb - 52;
    mant = (u + (1ull << (sh - 1))) >> sh;
    if (mant >> 53) {  // rounding carried into a new leading bit
      mant >>= 1;
      ++msb;
    }
  } else {
    mant = u << (52 - msb);
  }
  const int be = msb + E + 1023;
  if (be <= 0 || be >= 2047) return ldexp((double)Y, E);
  return __longlong_as_double((long long)((s << 63) | ((unsigned long long)be << 52) | (mant & ((1ull << 52) - 1))));
}

// D[i, j] -= sum_c A_real[i, c] B_real[j, c] (exact to the truncation above)
// for i < rows, j < cols; D row-major doubles, leading dimension ldd.
__global__ void __launch_bounds__(192, 1) k_tc_update_f64(const __grid_constant__ CUtensorMap tmA,
                                                          const __grid_constant__ CUtensorMap tmB,
                                                          double *__restrict__ D, long ldd, int rows, int cols,
                                                          int natoms, int k2p, const int *__restrict__ eA,
                                                          const int *__restrict__ fB, int *err) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char *base = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                          ~static_cast<uintptr_t>(1023));
  const uint32_t sA = smem_u32(base);
  const uint32_t sB = sA + FB_MAX_ATOMS * FB_ATOM_A;
  uint64_t *bars = reinterpret_cast<uint64_t *>(base + FB_MAX_ATOMS * (FB_ATOM_A + FB_ATOM_B));
  uint32_t *tslot = reinterpret_cast<uint32_t *>(bars + 2);
  int *sf = reinterpret_cast<int *>(bars + 4);  // FB_BN column exponents
  const uint32_t full = smem_u32(bars), done = full + 8;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * FB_BM, n0 = blockIdx.x * FB_BN;

  if (threadIdx.x == 0) {
    mbar_init(full, 1);
    mbar_init(done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (threadIdx.x < FB_BN) sf[threadIdx.x] = (n0 + (int)threadIdx.x < cols) ? fB[n0 + threadIdx.x] : 0;
  if (warp == 1) tmem_alloc(smem_u32(tslot), 512);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;

  if (warp == 0) {
    if (lane == 0) {
      mbar_expect_tx(full, (uint32_t)natoms * (FB_ATOM_A + FB_ATOM_B));
      for (int a = 0; a < natoms; ++a) {
        tma_load_2d(sA + a * FB_ATOM_A, &tmA, a * 64, m0, full);
        tma_load_2d(sB + a * FB_ATOM_B, &tmB, a * 64, n0, full);
      }
      // Drain: the copies have landed before the CTA can exit.
      if (!mbar_wait(full, 0)) atomicExch(err, 11);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      if (mbar_wait(full, 0)) {
        tc_fence_after();
        for (int l = 2; l <= FB_LMAX; ++l) {
          const uint32_t dcol = tmem + (uint32_t)((l - 2) * FB_BN);
          bool first = true;
          for (int p = 1; p <= FB_S; ++p) {
            const int q = l - p;
            if (q < 1 || q > FB_S) continue;
            for (int kc = 0; kc < k2p; kc += 16) {
              const int oa = (p - 1) * k2p + kc, ob = (q - 1) * k2p + kc;
              const uint64_t ad = sw128_desc(sA + (oa >> 6) * FB_ATOM_A + (oa & 63) * 2);
              const uint64_t bd = sw128_desc(sB + (ob >> 6) * FB_ATOM_B + (ob & 63) * 2);
              mma_bf16(dcol, ad, bd, kIdescBF16, first ? 0u : 1u);
              first = false;
            }
          }
        }
      } else {
        atomicExch(err, 12);
      }
      mma_commit(done);
    }
    __syncwarp();
  } else {
    const int q = warp & 3;
    const int row = m0 + q * 32 + lane;
    const bool rin = row < rows;
    const int ea = rin ? eA[row] : 0;
    double *drow = D + (size_t)row * ldd;
    // Chunk c of this thread's row segment: 16 doubles. Loads run one chunk
    // ahead (the first while the MMAs run).
    double2 cur[8], nxt[8];
    auto load_chunk = [&](int c, double2 *dst) {
      const int col0 = n0 + c * 16;
#pragma unroll
      for (int u = 0; u < 8; ++u)
        dst[u] = (rin && col0 + 16 <= cols) ? reinterpret_cast<const double2 *>(drow + col0)[u]
                                            : make_double2(0.0, 0.0);
    };
    load_chunk(0, cur);
    const bool ok = __all_sync(0xffffffffu, mbar_wait(done, 0));
    tc_fence_after();
    if (!ok) {
      if (lane == 0) atomicExch(err, 13);
    } else {
#pragma unroll
      for (int c = 0; c < FB_BN / 16; ++c) {
        if (c + 1 < FB_BN / 16) load_chunk(c + 1, nxt);
        long long Y[16];
#pragma unroll
        for (int u = 0; u < 16; ++u) Y[u] = 0;
#pragma unroll
        for (int l = 2; l <= FB_LMAX; ++l) {
          float v[16];
          tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)((l - 2) * FB_BN + c * 16), v);
#pragma unroll
          for (int u = 0; u < 16; ++u) {
            const long long C = f2i_exact(v[u]);
            Y[u] += l < FB_LMAX ? (C << (FB_B * (FB_LMAX - 1 - l))) : ((C + 64) >> FB_B);
          }
        }
        const int col0 = n0 + c * 16;
        if (rin) {
          if (col0 + 16 <= cols) {
            double2 *p = reinterpret_cast<double2 *>(drow + col0);
#pragma unroll
            for (int u = 0; u < 8; ++u) {
              double2 x = cur[u];
              x.x -= i64_scaled(Y[2 * u], ea + sf[c * 16 + 2 * u] - FB_B * (FB_LMAX - 1));
              x.y -= i64_scaled(Y[2 * u + 1], ea + sf[c * 16 + 2 * u + 1] - FB_B * (FB_LMAX - 1));
              p[u] = x;
            }
          } else {
            for (int u = 0; u < 16; ++u)
              if (col0 + u < cols) drow[col0 + u] -= i64_scaled(Y[u], ea + sf[c * 16 + u] - FB_B * (FB_LMAX - 1));
          }
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) cur[u] = nxt[u];
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, 512);
  }
}

PFN_cuTensorMapEncodeTiled_v12000 g_enc = nullptr;
std::once_flag g_enc_once;

cudaError_t make_map_bf16(CUtensorMap *m, const void *base, long rows, int K, long ldk, int box_rows) {
  std::call_once(g_enc_once, [] {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_enc = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  });
  if (!g_enc) return cudaErrorNotSupported;
  const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)ldk * 2};
  const cuuint32_t box[2] = {64, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = g_enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

}  // namespace

int f64tc_max_k() { return 32; }

size_t f64tc_op_cols() { return (size_t)FB_MAX_ATOMS * 64; }

cudaError_t launch_f64tc_update(Handle *h, int f, int k, double2 *M, const double2 *A, const double2 *W) {
  const long n = h->n, rows = n + h->E;
  const long cols = 2 * (n + 1);
  if (k < 1 || k > f64tc_max_k()) return cudaErrorInvalidValue;
  const int k2p = (2 * k + 15) / 16 * 16;
  const int kop = (FB_S * k2p + 63) / 64 * 64;
  const int natoms = kop / 64;
  const long ldk = (long)f64tc_op_cols();
  // operand rows have pitch ldk; each update fills its rows up to the pitch
  k_slice_A<<<(unsigned)((rows + 127) / 128), 128, 0, h->stream>>>(
      A, rows, rows, k, k2p, (int)ldk, static_cast<__nv_bfloat16 *>(h->d_A16), h->d_eA);
  k_slice_B<<<(unsigned)((cols + 127) / 128), 128, 0, h->stream>>>(
      W, h->ldm, cols, k, k2p, (int)ldk, static_cast<__nv_bfloat16 *>(h->d_B16), h->d_fB);
  CUtensorMap ma, mb;
  cudaError_t e;
  if ((e = make_map_bf16(&ma, h->d_A16, h->a16_rows, kop, ldk, FB_BM)) != cudaSuccess) return e;
  if ((e = make_map_bf16(&mb, h->d_B16, h->b16_rows, kop, ldk, FB_BN)) != cudaSuccess) return e;
  if ((e = cudaFuncSetAttribute(k_tc_update_f64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FB_SMEM)) !=
      cudaSuccess)
    return e;
  dim3 g((unsigned)((cols + FB_BN - 1) / FB_BN), (unsigned)((rows + FB_BM - 1) / FB_BM));
  cudaEvent_t t0 = timing_mark(h);
  k_tc_update_f64<<<g, 192, FB_SMEM, h->stream>>>(ma, mb, reinterpret_cast<double *>(M), 2 * h->ldm, (int)rows,
                                                  (int)cols, natoms, k2p, h->d_eA, h->d_fB, h->d_tc_err);
  const double cells = (double)rows * (double)(n + 1);
  timing_close(h, t0, T_UPDATE, 8.0 * k * cells, 2.0 * 16.0 * cells + 2.0 * kop * ((double)rows + (double)cols),
               0.0);
  h->nlaunch += 3;
  (void)f;
  return cudaGetLastError();
}

}  // namespace pngf
