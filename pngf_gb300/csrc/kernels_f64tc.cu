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
//    K stay integers below 2^22 (k <= 32), so the FP32 accumulation in TMEM is
//    exact. Pairs with p + q = l share one accumulator per level l = 2..8 (28
//    pairs in 7 TMEM accumulators); pairs with p + q > 8 are dropped, an error
//    below 2^-50 of the row/column scales -- finer than FP64 GEMM rounding;
//  * the epilogue recombines the levels exactly in integers,
//    Y = sum_l C_l 2^(7(7-l)), builds Y 2^(e+f-49) as a double from its bits
//    and subtracts it from M: one FP64 add per element.
//
// Kernel k_tc_update_f64 is persistent: one CTA per SM walks a contiguous
// range of 128-row x 32-double-column tiles of M (row-block major). Warp 0
// issues the copies: the operand tiles, which the slicing kernels write in
// HBM in the MMA's unswizzled core-matrix layout, by plain bulk copies (the A
// row block stays in shared memory across its column tiles, B tiles are
// double-buffered), and each tile of M by TMA into a ring of up to three
// shared-memory slots ahead of its epilogue (the staging that hides HBM
// latency). Warp 1 issues the tcgen05.mma.kind::f16 (M=128, K=16) chains into
// one of two TMEM accumulator sets (7 levels x 32 columns each), two groups
// of 8 epilogue warps take alternate tiles (one group's FP64 subtractions
// overlap the other group's integer work) and update the staged tile in
// shared memory, and warp 2 writes each finished tile back with a TMA store.
// M thus moves between HBM and the SM only in whole swizzled tiles. Every
// wait is bounded; on timeout the kernel records an error code, drains its
// own copies, frees its TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdint>
#include <mutex>

#include "bounds.cuh"
#include "pngf_internal.h"
#include "tc_common.cuh"

namespace pngf {

namespace {

using namespace tc;

constexpr int FB_BM = 128;            // rows of M per tile (MMA M)
constexpr int FB_BN = 32;             // double columns of M per tile (MMA N)
constexpr int FB_S = 7;               // slices per operand
constexpr int FB_B = 7;               // bits per slice
constexpr int FB_LMAX = 8;            // highest level kept (p + q <= 8)
constexpr int FB_NLEV = FB_LMAX - 1;  // levels 2..8
constexpr int FB_ACC = FB_NLEV * FB_BN;  // TMEM columns of one accumulator set (224)
constexpr int FB_ACC_STRIDE = 256;       // TMEM column offset between the two sets
static_assert(FB_ACC <= FB_ACC_STRIDE && 2 * FB_ACC_STRIDE <= 512, "two accumulator sets in 512 TMEM columns");
constexpr int FB_MAX_K2P = 64;               // 2k padded to 16, k <= 32
constexpr int FB_BROWS = FB_S * FB_BN;       // B tile: the 7 slices of 32 output columns stacked along N
// bytes of an A tile (128 rows x 7 k2p) and of a B tile (224 rows x k2p), multiples of 1024
__host__ __device__ constexpr uint32_t fb_abytes(int k2p) { return (uint32_t)FB_BM * FB_S * k2p * 2; }
__host__ __device__ constexpr uint32_t fb_bbytes(int k2p) { return (uint32_t)FB_BROWS * k2p * 2; }
constexpr int FB_EPI_WARPS = 16;                   // two groups of 8 (one per parity of the tile)
constexpr int FB_GROUP_WARPS = FB_EPI_WARPS / 2;
constexpr int FB_MAX_ND = 3;  // staged tiles of M at most
constexpr int FB_DRING = 4;   // d_full / d_done barriers: even (two groups) and >= FB_MAX_ND
static_assert(FB_DRING % 2 == 0 && FB_DRING >= FB_MAX_ND, "tile barrier ring");
// mbarrier indices in the barrier block
constexpr int FB_BAR_A = 0, FB_BAR_BF = 2, FB_BAR_BE = 4, FB_BAR_ACCF = 6, FB_BAR_ACCE = 8, FB_BAR_DF = 10,
              FB_BAR_DD = FB_BAR_DF + FB_DRING, FB_BAR_DE = FB_BAR_DD + FB_DRING, FB_NBARS = FB_BAR_DE + FB_DRING;
static_assert(FB_NBARS * 8 + 4 <= 256, "barriers and the TMEM address fit the reserved 256 bytes");
constexpr int FB_THREADS = 96 + 32 * FB_EPI_WARPS;  // producer, MMA and store warps + epilogue
constexpr uint32_t FB_DBOX = FB_BM * 128;           // 128 rows x 16 doubles of M (one TMA box)
constexpr uint32_t FB_DTILE = 2 * FB_DBOX;          // a 128 x 32-double tile of M
// Dynamic shared memory for the A tile, nb B tiles and nd staged tiles of M.
constexpr size_t fb_smem(int k2p, int nb, int nd) {
  return 1024 + fb_abytes(k2p) + (size_t)nb * fb_bbytes(k2p) + (size_t)nd * FB_DTILE + 256;
}

// kind::f16 instruction descriptor: D f32, A and B bf16, K-major, M = 128, N = n.
__host__ __device__ constexpr uint32_t idesc_bf16(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(FB_BM >> 4) << 24);
}

// Power-of-two row / column scale e with max |x| 2^-e < 1, from the largest
// |x|'s bit pattern (non-negative doubles order like unsigned integers).
__device__ __forceinline__ int scale_exp_bits(unsigned long long mb) {
  if (mb == 0) return 0;
  const int be = (int)(mb >> 52);
  if (be > 0) return be - 1022;                        // ilogb + 1
  return (63 - __clzll((long long)mb)) - 1074 + 1;     // subnormal maximum
}

__device__ __forceinline__ unsigned long long abs_bits(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
}

// The 7 balanced base-128 digits of x 2^-e (|x| 2^-e < 1), on the integer
// pipes: S = x 2^(49-e) rounded to the nearest integer (ties to even), then
// S = sum_p a_p 2^(49-7p) with each digit rounded from the top (a_1 in
// [-128, 128], the others in [-64, 64]). The remainder dropped below the last
// digit is at most 2^-50 of the scale.
__device__ __forceinline__ void digits7(double x, int e, int *a) {
  const long long b = __double_as_longlong(x);
  const int be = (int)((b >> 52) & 0x7FF);
  const unsigned long long frac = (unsigned long long)b & ((1ull << 52) - 1);
  const unsigned long long m = be ? (frac | (1ull << 52)) : frac;
  const int sh = (be ? be : 1) - 1075 + 49 - e;  // x 2^(49-e) = m 2^sh
  unsigned long long q;
  if (sh >= 0) {
    q = m << sh;
  } else if (sh <= -64) {
    q = 0;
  } else {
    const int s = -sh;
    q = m >> s;
    const unsigned long long rem = m & ((1ull << s) - 1), half = 1ull << (s - 1);
    if (rem > half || (rem == half && (q & 1))) ++q;
  }
  long long S = b < 0 ? -(long long)q : (long long)q;
#pragma unroll
  for (int p = 0; p < FB_S - 1; ++p) {
    const int t = FB_B * (FB_S - 1 - p);  // 42, 35, ..., 7
    const long long d = (S + (1ll << (t - 1))) >> t;
    a[p] = (int)d;
    S -= d << t;
  }
  a[FB_S - 1] = (int)S;
}

// Operand tiles are stored in HBM exactly as the MMA reads them from shared
// memory, so that one plain bulk copy moves a whole tile: the K-major
// canonical layout without swizzle, 8-row x 8-element core matrices of 128
// contiguous bytes, the core matrices of one 8-element K chunk stacked along
// the rows (8-row groups 128 B apart), K chunks one after the other. Element
// (r, kk) of a tile with R rows sits at (kk / 8) * 8R + (r / 8) * 64 +
// (r % 8) * 8 + kk % 8.
__device__ __forceinline__ size_t core_off(int r, int kk, int R) {
  return (size_t)(kk >> 3) * (size_t)(8 * R) + (size_t)(r >> 3) * 64 + (size_t)(r & 7) * 8 + (kk & 7);
}

// A_op: for each 128-row block of M's rows, a 128 x 7*k2p tile holding the
// slices of the interleaved real rows of A[i, :], slice p at K columns
// [p*k2p, p*k2p + 2k), zeros elsewhere; rows from `rows` up to `arows` (the
// last block's padding) are zeros. One warp per row, lanes over the values.
__global__ void k_slice_A(const double2 *__restrict__ A, long lda, long rows, long arows, int k, int k2p,
                          __nv_bfloat16 *__restrict__ Aop, int *__restrict__ eA) {
  const long i = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= arows) return;
  const int kp = FB_S * k2p;
  __nv_bfloat16 *tile = Aop + (size_t)(i / FB_BM) * FB_BM * kp;
  const int r = (int)(i % FB_BM);
  if (i >= rows) {
    for (int kk = lane; kk < kp; kk += 32) tile[core_off(r, kk, FB_BM)] = __float2bfloat16_rn(0.f);
    return;
  }
  unsigned long long mb = 0;
  for (int c = lane; c < k; c += 32) {
    const double2 a = A[(size_t)c * lda + i];
    mb = max(mb, max(abs_bits(a.x), abs_bits(a.y)));
  }
  for (int o = 16; o; o >>= 1) mb = max(mb, __shfl_xor_sync(0xffffffffu, mb, o));
  const int e = scale_exp_bits(mb);
  if (lane == 0) eA[i] = e;
  for (int v = lane; v < 2 * k; v += 32) {
    const double2 a = A[(size_t)(v >> 1) * lda + i];
    int d[FB_S];
    digits7((v & 1) ? a.y : a.x, e, d);
#pragma unroll
    for (int p = 0; p < FB_S; ++p) tile[core_off(r, p * k2p + v, FB_BM)] = __int2bfloat16_rn(d[p]);
  }
  for (int v = 2 * k + lane; v < k2p; v += 32)  // padding of each slice
    for (int p = 0; p < FB_S; ++p) tile[core_off(r, p * k2p + v, FB_BM)] = __float2bfloat16_rn(0.f);
}

__device__ __forceinline__ double2 ld_c(const double2 *p) { return *p; }
__device__ __forceinline__ double2 ld_c(const float2 *p) {
  const float2 v = *p;
  return make_double2(v.x, v.y);
}

// B_op for output column j' (j' = 2j: real part, 2j+1: imaginary, of column
// j of the product; W is k x ldw, row-major complex, row c taken from row
// rowidx[c] of W when rowidx is given). Column tile c = j' / 32 is a 224 x k2p
// tile (same layout as A's) in which the 7 slices of its 32 output columns
// are stacked along N: slice q of column j' is row (q - 1) * 32 + j' % 32,
// its 2k K entries then zeros. A tile's MMA with A-slice p then takes the rows
// of slices 1 .. 8 - p in one instruction (N = (8 - p) * 32) and lands slice q
// in TMEM columns of level p + q. Columns from ncols2 up to the end of the
// last tile are zeros. One warp per output column, lanes over the values.
template <typename TIN>
__global__ void k_slice_B(const TIN *__restrict__ W, long ldw, const int *__restrict__ rowidx, long rowlim,
                          long ncols2, long bcols, int k, int k2p, __nv_bfloat16 *__restrict__ Bop,
                          int *__restrict__ fB) {
  const long jp = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (jp >= bcols) return;
  __nv_bfloat16 *tile = Bop + (size_t)(jp / FB_BN) * FB_BROWS * k2p;
  const int n0 = (int)(jp % FB_BN);  // row of slice 1; slice q at row n0 + (q - 1) * 32
  if (jp >= ncols2) {
    for (int v = lane; v < k2p; v += 32)
      for (int q = 0; q < FB_S; ++q) tile[core_off(n0 + q * FB_BN, v, FB_BROWS)] = __float2bfloat16_rn(0.f);
    return;
  }
  const long j = jp >> 1;
  const bool im = jp & 1;
  unsigned long long mb = 0;
  for (int c = lane; c < k; c += 32) {
    const long rc = rowidx ? rowidx[c] : c;
    if (!PNGF_BOUNDS_OK(rc >= 0 && rc < rowlim, kBoundsRowIdx, rc, j)) continue;
    const double2 w = ld_c(W + (size_t)rc * ldw + j);
    mb = max(mb, max(abs_bits(w.x), abs_bits(w.y)));
  }
  for (int o = 16; o; o >>= 1) mb = max(mb, __shfl_xor_sync(0xffffffffu, mb, o));
  const int f = scale_exp_bits(mb);
  if (lane == 0) fB[jp] = f;
  for (int v = lane; v < 2 * k; v += 32) {
    const int c = v >> 1;
    const long rc = rowidx ? rowidx[c] : c;
    const double2 w = PNGF_BOUNDS_OK(rc >= 0 && rc < rowlim, kBoundsRowIdx, rc, j) ? ld_c(W + (size_t)rc * ldw + j)
                                                                                  : make_double2(0.0, 0.0);
    // Re out: Re A Re W - Im A Im W; Im out: Re A Im W + Im A Re W
    const double x = (v & 1) ? (im ? w.x : -w.y) : (im ? w.y : w.x);
    int d[FB_S];
    digits7(x, f, d);
#pragma unroll
    for (int q = 0; q < FB_S; ++q) tile[core_off(n0 + q * FB_BN, v, FB_BROWS)] = __int2bfloat16_rn(d[q]);
  }
  for (int v = 2 * k + lane; v < k2p; v += 32)
    for (int q = 0; q < FB_S; ++q) tile[core_off(n0 + q * FB_BN, v, FB_BROWS)] = __float2bfloat16_rn(0.f);
}

// Exact bit pattern offset of a float holding an integer of magnitude below
// 2^22 after adding 1.5 * 2^23 (the integer lands in the low mantissa bits).
constexpr int kMagicBits = 0x4B400000;
__device__ __forceinline__ int fbits(float v) { return __float_as_int(v + 12582912.0f); }

// Y * 2^E as a double, built from the bits on the integer pipes (round half
// up to 53 bits), |Y| < 2^63. Entirely integer and branch-free, so that no
// FP64 instruction besides the subtraction of the result is issued (GB300's
// FP64 pipe executes 2 lanes per clock per SM). Results below the normal
// range (|Y 2^E| < 2^-1022) flush to zero and results above it become
// infinities; M's entries are many orders of magnitude inside that range.
__device__ __forceinline__ double i64_scaled(long long Y, int E) {
  const unsigned long long s = (unsigned long long)Y & (1ull << 63);
  const unsigned long long u = (unsigned long long)(Y < 0 ? -Y : Y);
  const int lz = __clzll((long long)u);  // 64 for Y = 0
  const unsigned long long nrm = u << (lz & 63);                  // leading bit at 63
  const unsigned long long mant = (nrm >> 11) + ((nrm >> 10) & 1);  // 2^52 .. 2^53
  const int be = 63 - lz + E + 1023;
  // (be - 1) 2^52 + mant: a carry of the rounding into 2^53 raises the exponent
  const unsigned long long mag = u == 0 || be <= 0 ? 0ull
                                 : be >= 2047      ? 0x7FF0000000000000ull
                                                   : ((unsigned long long)(be - 1) << 52) + mant;
  return __longlong_as_double((long long)(s | mag));
}

// D[i, j] -= sum_c A_real[i, c] B_real[j, c] for i < rows, j < cols; D is
// M viewed as row-major doubles, reached only through the tensor map tmD
// (128 x 16-double boxes, 128-byte swizzle). ncb = column tiles per row
// block, ntiles = total tiles, Aop / Bop = the operand tiles (k2p: 2k padded to 16),
// nb = B-tile buffers (1 or 2), nd = staged tiles of M (1 to 3).
//
// Tiles of M travel by TMA: the producer loads tile t into a shared-memory
// slot (a ring of nd) ahead of its epilogue, the epilogue group of the tile's
// parity updates the slot in place (thread = row, 16 doubles each,
// conflict-free under the swizzle) and the store warp writes the slot back
// with a TMA store, then frees the slot.
__global__ void __launch_bounds__(FB_THREADS, 1)
    k_tc_update_f64(const __nv_bfloat16 *__restrict__ Aop, const __nv_bfloat16 *__restrict__ Bop,
                    const __grid_constant__ CUtensorMap tmD, int rows, int cols, int ncb, int ntiles, int k2p, int nb,
                    int nd, const int *__restrict__ eA, const int *__restrict__ fB, int *err) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char *base = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                          ~static_cast<uintptr_t>(1023));
  const uint32_t sA = smem_u32(base);
  const uint32_t a_bytes = fb_abytes(k2p), b_bytes = fb_bbytes(k2p);
  const uint32_t sB0 = sA + a_bytes;                      // B buffer b at sB0 + b * b_bytes
  const uint32_t dbase = a_bytes + (uint32_t)nb * b_bytes;  // byte offset of slot 0 from base (a multiple of 1024)
  const uint32_t sD0 = sA + dbase;
  uint64_t *bars = reinterpret_cast<uint64_t *>(base + dbase + (uint32_t)nd * FB_DTILE);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(bars + FB_NBARS);
  const uint32_t bar0 = smem_u32(bars);
  auto bar = [&](int i) { return bar0 + 8u * (uint32_t)i; };
  const uint32_t a_full = bar(FB_BAR_A), a_empty = bar(FB_BAR_A + 1);
  auto b_full = [&](int b) { return bar(FB_BAR_BF + b); };      // b < 2
  auto b_empty = [&](int b) { return bar(FB_BAR_BE + b); };
  auto acc_full = [&](int b) { return bar(FB_BAR_ACCF + b); };  // accumulator set b < 2
  auto acc_empty = [&](int b) { return bar(FB_BAR_ACCE + b); };
  // A tile of M: d_full(j) / d_done(j) with j = li % 4 (a multiple of the
  // group count and >= nd, so that a barrier is re-armed only after its last
  // phase has been waited for), d_empty by the shared-memory slot (li % nd).
  auto d_full = [&](int j) { return bar(FB_BAR_DF + j); };
  auto d_done = [&](int j) { return bar(FB_BAR_DD + j); };
  auto d_empty = [&](int s) { return bar(FB_BAR_DE + s); };
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  // this CTA's contiguous tile range
  const int t_begin = (int)(((long long)ntiles * blockIdx.x) / gridDim.x);
  const int t_end = (int)(((long long)ntiles * (blockIdx.x + 1)) / gridDim.x);

  if (threadIdx.x == 0) {
    mbar_init(a_full, 1);
    mbar_init(a_empty, 1);
    for (int b = 0; b < 2; ++b) {
      mbar_init(b_full(b), 1);
      mbar_init(b_empty(b), 1);
      mbar_init(acc_full(b), 1);
      mbar_init(acc_empty(b), FB_GROUP_WARPS);
    }
    for (int j = 0; j < FB_DRING; ++j) {
      mbar_init(d_full(j), 1);
      mbar_init(d_done(j), FB_GROUP_WARPS);
      mbar_init(d_empty(j), 1);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) tmem_alloc(smem_u32(tslot), 512);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;

  if (warp == 0) {
    if (lane == 0) {
      bool ok = true;
      int nA = 0, rb_loaded = -1, issuedB = 0, issuedD = 0;
      for (int t = t_begin; t < t_end && ok; ++t) {
        const int li = t - t_begin, rb = t / ncb, cb = t - rb * ncb;
        if (rb != rb_loaded) {
          if (nA > 0 && !mbar_wait(a_empty, (nA - 1) & 1)) { ok = false; break; }
          mbar_expect_tx(a_full, a_bytes);
          const unsigned char *src = reinterpret_cast<const unsigned char *>(Aop) + (size_t)rb * a_bytes;
          for (uint32_t o = 0; o < a_bytes; o += 16384)
            bulk_load(sA + o, src + o, min(16384u, a_bytes - o), a_full);
          rb_loaded = rb;
          ++nA;
        }
        const int bb = li % nb, j = li % FB_DRING;
        if (li >= nb && !mbar_wait(b_empty(bb), ((li / nb) - 1) & 1)) { ok = false; break; }
        mbar_expect_tx(b_full(bb), b_bytes);
        bulk_load(sB0 + bb * b_bytes, reinterpret_cast<const unsigned char *>(Bop) + (size_t)cb * b_bytes, b_bytes,
                  b_full(bb));
        ++issuedB;
        const int s = li % nd;
        if (li >= nd && !mbar_wait(d_empty(s), ((li / nd) - 1) & 1)) { ok = false; break; }
        mbar_expect_tx(d_full(j), FB_DTILE);
        tma_load_2d(sD0 + s * FB_DTILE, &tmD, cb * FB_BN, rb * FB_BM, d_full(j));
        tma_load_2d(sD0 + s * FB_DTILE + FB_DBOX, &tmD, cb * FB_BN + 16, rb * FB_BM, d_full(j));
        ++issuedD;
      }
      if (!ok) atomicExch(err, 21);
      // Drain the copies in flight before the CTA can exit.
      if (nA > 0 && !mbar_wait(a_full, (nA - 1) & 1)) atomicExch(err, 24);
      for (int li = issuedB > nb ? issuedB - nb : 0; li < issuedB; ++li)
        if (!mbar_wait(b_full(li % nb), (li / nb) & 1)) atomicExch(err, 24);
      for (int li = issuedD > nd ? issuedD - nd : 0; li < issuedD; ++li)
        if (!mbar_wait(d_full(li % FB_DRING), (li / FB_DRING) & 1)) atomicExch(err, 24);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      bool ok = true;
      int nA = 0, rb_have = -1;
      for (int t = t_begin; t < t_end; ++t) {
        const int li = t - t_begin, rb = t / ncb;
        if (rb != rb_have) {
          if (!mbar_wait(a_full, nA & 1)) { ok = false; break; }
          rb_have = rb;
          ++nA;
        }
        const int b = li & 1, bb = li % nb;
        if (!mbar_wait(b_full(bb), (li / nb) & 1)) { ok = false; break; }
        if (li >= 2 && !mbar_wait(acc_empty(b), ((li >> 1) - 1) & 1)) { ok = false; break; }
        tc_fence_after();
        const uint32_t sB = sB0 + bb * b_bytes;
        const uint32_t acc = tmem + (uint32_t)(b * FB_ACC_STRIDE);
        // A-slice p against B-slices 1 .. 8-p in one MMA (N = (8-p) * 32): the
        // product with slice q lands in the columns of level l = p + q (levels
        // 2..8 at columns 32 (l-2)). p = 1 covers every level and starts them.
        for (int p = 1; p <= FB_S; ++p) {
          const uint32_t dcol = acc + (uint32_t)((p - 1) * FB_BN);
          const uint32_t idesc = idesc_bf16((FB_LMAX - p) * FB_BN);
          for (int kc = 0; kc < k2p; kc += 16) {
            const int oa = (p - 1) * k2p + kc;
            // K chunks of 8 elements are 8 * rows * 2 bytes apart, 8-row groups 128 bytes
            const uint64_t ad = plain_desc(sA + (uint32_t)(oa >> 3) * (8 * FB_BM * 2), 8 * FB_BM * 2, 128);
            const uint64_t bd = plain_desc(sB + (uint32_t)(kc >> 3) * (8 * FB_BROWS * 2), 8 * FB_BROWS * 2, 128);
            mma_bf16(dcol, ad, bd, idesc, (p > 1 || kc > 0) ? 1u : 0u);
          }
        }
        mma_commit(b_empty(bb));
        mma_commit(acc_full(b));
        const bool last_of_rb = (t + 1 == t_end) || ((t + 1) / ncb != rb);
        if (last_of_rb) mma_commit(a_empty);
      }
      if (!ok) atomicExch(err, 22);
    }
    __syncwarp();
  } else if (warp == 2) {
    if (lane == 0) {
      bool ok = true;
      for (int t = t_begin; t < t_end; ++t) {
        const int li = t - t_begin, rb = t / ncb, cb = t - rb * ncb, s = li % nd;
        if (!mbar_wait(d_done(li % FB_DRING), (li / FB_DRING) & 1)) { ok = false; break; }
        const uint32_t sd = sD0 + s * FB_DTILE;
        tma_store_2d(&tmD, sd, cb * FB_BN, rb * FB_BM);  // rows / columns past M are clipped
        if (cb * FB_BN + 16 < cols) tma_store_2d(&tmD, sd + FB_DBOX, cb * FB_BN + 16, rb * FB_BM);
        bulk_commit();
        bulk_wait_read_all();
        mbar_arrive(d_empty(s));
      }
      bulk_wait_all();
      if (!ok) atomicExch(err, 25);
    }
    __syncwarp();
  } else {
    // Two groups of 8 warps take alternate tiles (group g: local tiles g, g+2,
    // ...) with accumulator set g, so that one group's FP64 subtractions
    // overlap the other group's TMEM reads and integer work. A warp covers 32
    // rows (its TMEM lane quarter) x 16 columns (one TMA box of the tile).
    const int ew = warp - 3;          // 0..15
    const int g = ew / FB_GROUP_WARPS;
    const int half = (ew >> 2) & 1;   // which 16 columns of the tile
    const int q = warp & 3;           // TMEM lanes 32q .. 32q+31
    const int r = q * 32 + lane;      // row of the tile
    // this thread's 16 doubles: row r of box `half`, 16-byte chunks 0..7
    const uint32_t rowoff = dbase + (uint32_t)half * FB_DBOX + (uint32_t)r * 128;
    bool ok = true;
    for (int t = t_begin + g; t < t_end; t += 2) {
      const int li = t - t_begin, rb = t / ncb, cb = t - rb * ncb;
      const int s = li % nd;  // li & 1 == g selects the accumulator set
      const int row = rb * FB_BM + r;
      const int col0 = cb * FB_BN + half * 16;  // < ncb * 32, within the padded scale arrays
      const int ea = row < rows ? eA[row] : 0;
      ok = __all_sync(0xffffffffu, mbar_wait(acc_full(g), (li >> 1) & 1));
      if (!ok) break;
      tc_fence_after();
      // Levels in pairs: P = C_l * 2^7 + C_{l+1} is an exact int32;
      // Y = P23 2^28 + P45 2^14 + P67 + round(C8 / 2^7). The level values are
      // the float bits minus kMagicBits; the offsets are taken off once per
      // pair (wrapping 32-bit arithmetic, exact since each P fits in int32).
      long long Y[16];
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        // the seven level loads of 8 columns in flight at once, one wait
        const uint32_t tbase =
            tmem + (uint32_t)(g * FB_ACC_STRIDE) + ((uint32_t)(q * 32) << 16) + (uint32_t)(half * 16 + c * 8);
        uint32_t v[FB_NLEV][8];
#pragma unroll
        for (int l = 0; l < FB_NLEV; ++l) tmem_ld8_nowait(tbase + (uint32_t)(l * FB_BN), v[l]);
        tmem_wait_ld();
        if (c == 1) {
          // every level of the tile is in registers: the accumulator set is
          // free once every warp of the group has read it
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(acc_empty(g));
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          auto F = [&](int l) { return (unsigned)fbits(__uint_as_float(v[l][u])); };
          constexpr unsigned kPair = 129u * (unsigned)kMagicBits;
          const int p23 = (int)(F(0) * 128u + F(1) - kPair), p45 = (int)(F(2) * 128u + F(3) - kPair);
          const int p67 = (int)(F(4) * 128u + F(5) - kPair), r8 = (int)(F(6) - (unsigned)(kMagicBits - 64)) >> 7;
          Y[c * 8 + u] = ((long long)p23 << 28) + ((long long)p45 << 14) + (long long)(p67 + r8);
        }
      }
      int fb[16];
      const int4 *f4 = reinterpret_cast<const int4 *>(fB + col0);
#pragma unroll
      for (int w = 0; w < 4; ++w) {
        const int4 f = f4[w];
        fb[4 * w] = f.x;
        fb[4 * w + 1] = f.y;
        fb[4 * w + 2] = f.z;
        fb[4 * w + 3] = f.w;
      }
      ok = __all_sync(0xffffffffu, mbar_wait(d_full(li % FB_DRING), (li / FB_DRING) & 1));
      if (!ok) break;
      // Rows and columns past M hold the TMA's zero fill and Y = 0 there;
      // the store clips them.
      const int E0 = ea - FB_B * (FB_LMAX - 1);
      unsigned char *slot = base + rowoff + (size_t)s * FB_DTILE;
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        double2 *p = reinterpret_cast<double2 *>(slot + 16 * (u ^ (r & 7)));
        double2 x = *p;
        x.x -= i64_scaled(Y[2 * u], E0 + fb[2 * u]);
        x.y -= i64_scaled(Y[2 * u + 1], E0 + fb[2 * u + 1]);
        *p = x;
      }
      fence_proxy_async_smem();
      __syncwarp();
      if (lane == 0) mbar_arrive(d_done(li % FB_DRING));
    }
    if (!ok && lane == 0) atomicExch(err, 23);
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

// 2-D tensor map over M as row-major doubles: cols x rows, row pitch ldd
// doubles, 16 x 128 boxes, 128-byte swizzle (zero fill outside M).
cudaError_t make_map_f64(CUtensorMap *m, const double *base, long rows, long cols, long ldd) {
  std::call_once(g_enc_once, [] {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_enc = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  });
  if (!g_enc) return cudaErrorNotSupported;
  const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)ldd * 8};
  const cuuint32_t box[2] = {16, (cuuint32_t)FB_BM};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = g_enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, const_cast<double *>(base), dims, strides, box,
                           estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

int g_num_sms = 0;
int g_smem_optin = 0;

}  // namespace

int f64tc_max_k() { return 32; }

cudaError_t bounds_read_f64tc(long long out[4], bool reset) {
#ifdef PNGF_BOUNDS_CHECK
  return bounds_read_tu(out, reset);
#else
  (void)reset;
  for (int q = 0; q < 4; ++q) out[q] = 0;
  return cudaSuccess;
#endif
}

size_t f64tc_op_cols() { return (size_t)FB_S * FB_MAX_K2P; }

size_t f64tc_b_cols() { return FB_MAX_K2P; }

long f64tc_b_rows(long n) { return (2 * (n + 1) + FB_BN - 1) / FB_BN * FB_BROWS; }

namespace {

// D[i, j] -= sum_c A[i, c] B[c, j] (complex, FP64-accurate) for i < drows
// and complex columns j < dcols2 / 2, with k <= f64tc_max_k(): D row-major
// doubles with pitch ldd, A column-major (lda), B row-major complex (ldb;
// complex64 when b32), its row c taken from row browidx[c] when given. On
// the lane's operand scratch and stream.
cudaError_t f64tc_gemm(Handle *h, int f, int k, double *D, long drows, long dcols2, long ldd, const double2 *A,
                       long lda, const void *B, bool b32, long ldb, const int *browidx, bool timed,
                       bool chain = true) {
  if (k < 1 || k > f64tc_max_k()) return cudaErrorInvalidValue;
  const int k2p = (2 * k + 15) / 16 * 16;
  const int nrb = (int)((drows + FB_BM - 1) / FB_BM), ncb = (int)((dcols2 + FB_BN - 1) / FB_BN);
  const long arows = (long)nrb * FB_BM, bcols = (long)ncb * FB_BN;
  // the operand buffers hold a16_rows x f64tc_op_cols() and b16_rows x f64tc_b_cols() elements
  if (arows > h->a16_rows || (long)ncb * FB_BROWS > h->b16_rows) return cudaErrorInvalidValue;
  Lane &L = lane_of(h, f);
  cudaStream_t st = lane_stream(h, f);
  __nv_bfloat16 *A16 = static_cast<__nv_bfloat16 *>(L.A16), *B16 = static_cast<__nv_bfloat16 *>(L.B16);
  k_slice_A<<<(unsigned)((arows + 3) / 4), 128, 0, st>>>(A, lda, drows, arows, k, k2p, A16, L.eA);
  const long rowlim = browidx ? h->n : k;  // rows a gathered B row may come from (state rows), else B's own
  if (b32)
    k_slice_B<float2><<<(unsigned)((bcols + 3) / 4), 128, 0, st>>>(static_cast<const float2 *>(B), ldb, browidx,
                                                                    rowlim, dcols2, bcols, k, k2p, B16, L.fB);
  else
    k_slice_B<double2><<<(unsigned)((bcols + 3) / 4), 128, 0, st>>>(static_cast<const double2 *>(B), ldb, browidx,
                                                                     rowlim, dcols2, bcols, k, k2p, B16, L.fB);
  CUtensorMap md;
  cudaError_t e;
  if ((e = make_map_f64(&md, D, drows, dcols2, ldd)) != cudaSuccess) return e;
  if (g_num_sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&g_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (g_num_sms <= 0) g_num_sms = 1;
  }
  // Staged tiles of M hide HBM latency and a second B buffer keeps the MMAs
  // ahead of the epilogue: three tiles and two B buffers when they fit
  // (k <= 24), else two and two, else one B buffer.
  static const int kShapes[5][2] = {{2, 3}, {2, 2}, {1, 2}, {2, 1}, {1, 1}};
  int nb = 1, nd = 1;
  for (const auto &sh : kShapes)
    if (fb_smem(k2p, sh[0], sh[1]) <= (size_t)g_smem_optin) {
      nb = sh[0];
      nd = sh[1];
      break;
    }
  const size_t smem = fb_smem(k2p, nb, nd);
  if (smem > (size_t)g_smem_optin) return cudaErrorInvalidValue;
  if ((e = cudaFuncSetAttribute(k_tc_update_f64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
      cudaSuccess)
    return e;
  const int ntiles = nrb * ncb;
  const int grid = persistent_grid(h, ntiles, g_num_sms);
  if (timed && chain && (e = chain_update_wait(h, f, st)) != cudaSuccess) return e;  // the M update: one lane at a time
  cudaEvent_t t0 = timed ? timing_mark(h, st) : nullptr;
  k_tc_update_f64<<<grid, FB_THREADS, smem, st>>>(A16, B16, md, (int)drows, (int)dcols2, ncb, ntiles, k2p, nb, nd,
                                                  L.eA, L.fB, h->d_tc_err);
  if (timed && chain && (e = chain_update_done(h, f, st)) != cudaSuccess) return e;
  if (timed) {
    const double cells = (double)drows * (double)(dcols2 / 2);
    timing_close(h, t0, T_UPDATE, 8.0 * k * cells,
                 2.0 * 16.0 * cells + 2.0 * FB_S * k2p * ((double)drows + (double)dcols2), 0.0, st);
  }
  h->nlaunch += 3;
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_f64tc_update(Handle *h, int f, int k, double2 *M, const double2 *A, const double2 *W) {
  const long n = h->n, rows = n + h->E;
  // the inner dimension in pieces of at most f64tc_max_k(): each piece's
  // product is exact and rounded once into M (as a K-blocked DGEMM rounds
  // once per block); A and W are copies, so later pieces see the same operands.
  // Updates in pieces (k = 32 tile shapes) keep the frequency lanes concurrent.
  const bool chain = k <= f64tc_max_k();
  for (int c0 = 0; c0 < k; c0 += f64tc_max_k()) {
    const int kc = std::min(k - c0, f64tc_max_k());
    const cudaError_t e = f64tc_gemm(h, f, kc, reinterpret_cast<double *>(M), rows, 2 * (n + 1), 2 * h->ldm,
                                     A + (size_t)c0 * rows, rows, W + (size_t)c0 * h->ldm, false, h->ldm, nullptr,
                                     true, chain);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_f64tc_small(Handle *h, int f, int k, double2 *D, long drows, long ncols, long ldd,
                               const double2 *A, long lda, const double2 *B, long ldb) {
  for (int c0 = 0; c0 < k; c0 += f64tc_max_k()) {
    const int kc = std::min(k - c0, f64tc_max_k());
    const cudaError_t e = f64tc_gemm(h, f, kc, reinterpret_cast<double *>(D), drows, 2 * ncols, 2 * ldd,
                                     A + (size_t)c0 * lda, lda, B + (size_t)c0 * ldb, false, ldb, nullptr, false);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_f64tc_wgemm(Handle *h, int f, int k, const double2 *Vneg, const void *X, bool x32, long ldx,
                               const int *d_s, double2 *W) {
  // W[:, 0:N] -= Vneg X[s, 0:N], the inner dimension in pieces of at most f64tc_max_k()
  for (int c0 = 0; c0 < k; c0 += f64tc_max_k()) {
    const int kc = std::min(k - c0, f64tc_max_k());
    const cudaError_t e = f64tc_gemm(h, f, kc, reinterpret_cast<double *>(W), k, 2 * h->n, 2 * h->ldm,
                                     Vneg + (size_t)c0 * k, k, X, x32, ldx, d_s + c0, false);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace pngf
