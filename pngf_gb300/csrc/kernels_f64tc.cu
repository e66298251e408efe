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
// issues TMA loads (the A row-block stays in shared memory across its column
// tiles; B tiles are double-buffered; each tile of M is loaded into one of
// two shared-memory slots ahead of its epilogue), warp 1 issues the
// tcgen05.mma.kind::f16 (M=128, N=32, K=16) chains into one of two TMEM
// accumulator sets (7 levels x 32 columns each), 16 epilogue warps (four
// warpgroups, 8 columns each) drain one accumulator set while the MMAs fill
// the other and update the staged tile in shared memory, and warp 2 writes
// each finished tile back with a TMA store. M thus moves between HBM and the
// SM only in whole swizzled tiles. Every wait is bounded; on timeout the
// kernel records an error code, drains its own TMA copies, frees its TMEM
// and returns.
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

constexpr int FB_BM = 128;            // rows of M per tile (MMA M)
constexpr int FB_BN = 32;             // double columns of M per tile (MMA N)
constexpr int FB_S = 7;               // slices per operand
constexpr int FB_B = 7;               // bits per slice
constexpr int FB_LMAX = 8;            // highest level kept (p + q <= 8)
constexpr int FB_NLEV = FB_LMAX - 1;  // levels 2..8
constexpr int FB_ACC = FB_NLEV * FB_BN;  // TMEM columns of one accumulator set (224)
constexpr uint32_t FB_ATOM_A = FB_BM * 128;  // one 64-element K atom of the A tile
constexpr int FB_MAX_ATOMS = 7;              // K extent of A up to 448 (k <= 32)
constexpr int FB_BROWS = FB_S * FB_BN;       // B tile: the 7 slices of 32 output columns stacked along N
constexpr uint32_t FB_BTILE = FB_BROWS * 128;  // 224 rows x one 64-element K atom (2k <= 64)
constexpr int FB_EPI_WARPS = 16;
constexpr int FB_THREADS = 96 + 32 * FB_EPI_WARPS;  // producer, MMA and store warps + epilogue
constexpr uint32_t FB_DBOX = FB_BM * 128;           // 128 rows x 16 doubles of M (one TMA box)
constexpr uint32_t FB_DTILE = 2 * FB_DBOX;          // a 128 x 32-double tile of M
// Dynamic shared memory for natoms K atoms and nd staged tiles of M.
constexpr size_t fb_smem(int natoms, int nd) {
  return 1024 + (size_t)natoms * FB_ATOM_A + 2 * FB_BTILE + (size_t)nd * FB_DTILE + 256;
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

// A_op row i (i < rows): slices of the interleaved real row of A[i, :]. One
// warp per row, lanes over the 2k values. Row pitch ld; slice p at columns
// [p*k2p, p*k2p + 2k), zeros elsewhere.
__global__ void k_slice_A(const double2 *__restrict__ A, long lda, long rows, int k, int k2p, int ld,
                          __nv_bfloat16 *__restrict__ Aop, int *__restrict__ eA) {
  const long i = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= rows) return;
  unsigned long long mb = 0;
  for (int r = lane; r < k; r += 32) {
    const double2 a = A[(size_t)r * lda + i];
    mb = max(mb, max(abs_bits(a.x), abs_bits(a.y)));
  }
  for (int o = 16; o; o >>= 1) mb = max(mb, __shfl_xor_sync(0xffffffffu, mb, o));
  const int e = scale_exp_bits(mb);
  if (lane == 0) eA[i] = e;
  __nv_bfloat16 *row = Aop + (size_t)i * ld;
  for (int v = lane; v < 2 * k; v += 32) {
    const double2 a = A[(size_t)(v >> 1) * lda + i];
    int d[FB_S];
    digits7((v & 1) ? a.y : a.x, e, d);
#pragma unroll
    for (int p = 0; p < FB_S; ++p) row[p * k2p + v] = __int2bfloat16_rn(d[p]);
  }
  for (int c = lane; c < ld; c += 32) {  // padding of each slice and past the last one
    const int p = c / k2p, w = c - p * k2p;
    if (p >= FB_S || w >= 2 * k) row[c] = __float2bfloat16_rn(0.f);
  }
}

// B_op for output column j' < 2(N+1) (j' = 2j: real part, 2j+1: imaginary, of
// M[:, j]; W is k x ldw, row-major complex). The 7 slices of the 32 output
// columns of tile c = j' / 32 are stacked along N: slice q of column j' is row
// c * 224 + (q - 1) * 32 + j' % 32, its 2k K entries (then zeros) in a row
// of 64. A tile's MMA with A-slice p then takes rows of slices 1 .. 8 - p in one
// instruction (N = (8 - p) * 32) and lands slice q in TMEM columns of level
// p + q. One warp per output column, lanes over the 2k values.
__global__ void k_slice_B(const double2 *__restrict__ W, long ldw, long ncols2, int k,
                          __nv_bfloat16 *__restrict__ Bop, int *__restrict__ fB) {
  const long jp = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (jp >= ncols2) return;
  const long j = jp >> 1;
  const bool im = jp & 1;
  unsigned long long mb = 0;
  for (int r = lane; r < k; r += 32) {
    const double2 w = W[(size_t)r * ldw + j];
    mb = max(mb, max(abs_bits(w.x), abs_bits(w.y)));
  }
  for (int o = 16; o; o >>= 1) mb = max(mb, __shfl_xor_sync(0xffffffffu, mb, o));
  const int f = scale_exp_bits(mb);
  if (lane == 0) fB[jp] = f;
  __nv_bfloat16 *row = Bop + ((size_t)(jp / FB_BN) * FB_BROWS + (jp % FB_BN)) * 64;  // slice 1; slice q at +(q-1)*32 rows
  for (int v = lane; v < 2 * k; v += 32) {
    const double2 w = W[(size_t)(v >> 1) * ldw + j];
    // Re out: Re A Re W - Im A Im W; Im out: Re A Im W + Im A Re W
    const double x = (v & 1) ? (im ? w.x : -w.y) : (im ? w.y : w.x);
    int d[FB_S];
    digits7(x, f, d);
#pragma unroll
    for (int q = 0; q < FB_S; ++q) row[(size_t)q * FB_BN * 64 + v] = __int2bfloat16_rn(d[q]);
  }
  for (int c = 2 * k + lane; c < 64; c += 32)
    for (int q = 0; q < FB_S; ++q) row[(size_t)q * FB_BN * 64 + c] = __float2bfloat16_rn(0.f);
}

// Exact bit pattern offset of a float holding an integer of magnitude below
// 2^22 after adding 1.5 * 2^23 (the integer lands in the low mantissa bits).
constexpr int kMagicBits = 0x4B400000;
__device__ __forceinline__ int fbits(float v) { return __float_as_int(v + 12582912.0f); }

// Y * 2^E as a double, built from the bits on the integer pipe (round half
// up to 53 bits), |Y| < 2^63. Branch-free except for the fallback to ldexp
// outside the normal exponent range, so a thread's eight conversions
// interleave instead of running as eight dependent chains.
__device__ __forceinline__ double i64_scaled(long long Y, int E) {
  const unsigned long long s = (unsigned long long)(Y >> 63);  // 0 or all ones
  const unsigned long long u = ((unsigned long long)Y ^ s) - s;  // |Y|
  int msb = 63 - __clzll((long long)u);                         // -1 for Y = 0
  const int sh = max(msb - 52, 0);
  const unsigned long long up = (u + ((1ull << max(sh - 1, 0)) & (sh > 0 ? ~0ull : 0ull))) >> sh;
  unsigned long long mant = sh > 0 ? up : u << max(52 - msb, 0);
  const unsigned long long c = mant >> 53;  // rounding carried into a new leading bit
  mant >>= c;
  msb += (int)c;
  const int be = msb + E + 1023;
  const double r =
      __longlong_as_double((long long)((s << 63) | ((unsigned long long)be << 52) | (mant & ((1ull << 52) - 1))));
  if (u != 0 && (be <= 0 || be >= 2047)) return ldexp((double)Y, E);
  return u == 0 ? 0.0 : r;
}

// D[i, j] -= sum_c A_real[i, c] B_real[j, c] for i < rows, j < cols; D is
// M viewed as row-major doubles, reached only through the tensor map tmD
// (128 x 16-double boxes, 128-byte swizzle). ncb = column tiles per row
// block, ntiles = total tiles, natoms = 64-element K atoms of the operands,
// nd = staged tiles of M (1 or 2).
//
// Tiles of M travel by TMA: the producer loads tile t into a shared-memory
// slot ahead of its epilogue, the 16 epilogue warps update the slot in place
// (thread = row, 8 doubles each, conflict-free under the swizzle) and the
// store warp writes the slot back with a TMA store, then frees the slot.
__global__ void __launch_bounds__(FB_THREADS, 1)
    k_tc_update_f64(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                    const __grid_constant__ CUtensorMap tmD, int rows, int cols, int ncb, int ntiles, int natoms, int k2p,
                    int nd, const int *__restrict__ eA, const int *__restrict__ fB, int *err) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char *base = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                          ~static_cast<uintptr_t>(1023));
  const uint32_t sA = smem_u32(base);
  const uint32_t sB0 = sA + (uint32_t)natoms * FB_ATOM_A;  // B buffer b at sB0 + b * FB_BTILE
  const uint32_t dbase = (uint32_t)natoms * FB_ATOM_A + 2 * FB_BTILE;  // byte offset of slot 0 from base
  const uint32_t sD0 = sA + dbase;
  uint64_t *bars = reinterpret_cast<uint64_t *>(base + dbase + (uint32_t)nd * FB_DTILE);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(bars + 16);
  const uint32_t bar0 = smem_u32(bars);
  const uint32_t a_full = bar0, a_empty = bar0 + 8;
  auto b_full = [&](int b) { return bar0 + 16 + 8 * b; };
  auto b_empty = [&](int b) { return bar0 + 32 + 8 * b; };
  auto acc_full = [&](int b) { return bar0 + 48 + 8 * b; };
  auto acc_empty = [&](int b) { return bar0 + 64 + 8 * b; };
  auto d_full = [&](int s) { return bar0 + 80 + 8 * s; };   // tile of M landed in slot s
  auto d_done = [&](int s) { return bar0 + 96 + 8 * s; };   // epilogue finished slot s
  auto d_empty = [&](int s) { return bar0 + 112 + 8 * s; }; // store has read slot s
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
      mbar_init(acc_empty(b), FB_EPI_WARPS);
      mbar_init(d_full(b), 1);
      mbar_init(d_done(b), FB_EPI_WARPS);
      mbar_init(d_empty(b), 1);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) tmem_alloc(smem_u32(tslot), 512);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  const uint32_t a_bytes = (uint32_t)natoms * FB_ATOM_A;

  if (warp == 0) {
    if (lane == 0) {
      bool ok = true;
      int nA = 0, rb_loaded = -1, issuedB = 0, issuedD = 0;
      for (int t = t_begin; t < t_end && ok; ++t) {
        const int li = t - t_begin, rb = t / ncb, cb = t - rb * ncb;
        if (rb != rb_loaded) {
          if (nA > 0 && !mbar_wait(a_empty, (nA - 1) & 1)) { ok = false; break; }
          mbar_expect_tx(a_full, a_bytes);
          for (int a = 0; a < natoms; ++a) tma_load_2d(sA + a * FB_ATOM_A, &tmA, a * 64, rb * FB_BM, a_full);
          rb_loaded = rb;
          ++nA;
        }
        const int b = li & 1;
        if (li >= 2 && !mbar_wait(b_empty(b), ((li >> 1) - 1) & 1)) { ok = false; break; }
        mbar_expect_tx(b_full(b), FB_BTILE);
        tma_load_2d(sB0 + b * FB_BTILE, &tmB, 0, cb * FB_BROWS, b_full(b));
        ++issuedB;
        const int s = li % nd;
        if (li >= nd && !mbar_wait(d_empty(s), ((li / nd) - 1) & 1)) { ok = false; break; }
        mbar_expect_tx(d_full(s), FB_DTILE);
        tma_load_2d(sD0 + s * FB_DTILE, &tmD, cb * FB_BN, rb * FB_BM, d_full(s));
        tma_load_2d(sD0 + s * FB_DTILE + FB_DBOX, &tmD, cb * FB_BN + 16, rb * FB_BM, d_full(s));
        ++issuedD;
      }
      if (!ok) atomicExch(err, 21);
      // Drain the copies in flight before the CTA can exit.
      if (nA > 0 && !mbar_wait(a_full, (nA - 1) & 1)) atomicExch(err, 24);
      for (int li = issuedB > 2 ? issuedB - 2 : 0; li < issuedB; ++li)
        if (!mbar_wait(b_full(li & 1), (li >> 1) & 1)) atomicExch(err, 24);
      for (int li = issuedD > nd ? issuedD - nd : 0; li < issuedD; ++li)
        if (!mbar_wait(d_full(li % nd), (li / nd) & 1)) atomicExch(err, 24);
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
        const int b = li & 1;
        if (!mbar_wait(b_full(b), (li >> 1) & 1)) { ok = false; break; }
        if (li >= 2 && !mbar_wait(acc_empty(b), ((li >> 1) - 1) & 1)) { ok = false; break; }
        tc_fence_after();
        const uint32_t sB = sB0 + b * FB_BTILE;
        const uint32_t acc = tmem + (uint32_t)(b * 256);
        // A-slice p against B-slices 1 .. 8-p in one MMA (N = (8-p) * 32): the
        // product with slice q lands in the columns of level l = p + q (levels
        // 2..8 at columns 32 (l-2)). p = 1 covers every level and starts them.
        for (int p = 1; p <= FB_S; ++p) {
          const uint32_t dcol = acc + (uint32_t)((p - 1) * FB_BN);
          const uint32_t idesc = idesc_bf16((FB_LMAX - p) * FB_BN);
          for (int kc = 0; kc < k2p; kc += 16) {
            const int oa = (p - 1) * k2p + kc;
            const uint64_t ad = sw128_desc(sA + (oa >> 6) * FB_ATOM_A + (oa & 63) * 2);
            const uint64_t bd = sw128_desc(sB + kc * 2);
            mma_bf16(dcol, ad, bd, idesc, (p > 1 || kc > 0) ? 1u : 0u);
          }
        }
        mma_commit(b_empty(b));
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
        if (!mbar_wait(d_done(s), (li / nd) & 1)) { ok = false; break; }
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
    const int ew = warp - 3;          // 0..15
    const int part = ew >> 2;         // which 8 columns of the tile
    const int q = warp & 3;           // TMEM lanes 32q .. 32q+31
    const int r = q * 32 + lane;      // row of the tile
    // this thread's 8 doubles: box part / 2, 16-byte chunks c0 .. c0+3 of row r
    const uint32_t rowoff = dbase + (uint32_t)(part >> 1) * FB_DBOX + (uint32_t)r * 128;
    const int c0 = (part & 1) * 4;
    bool ok = true;
    for (int t = t_begin; t < t_end; ++t) {
      const int li = t - t_begin, rb = t / ncb, cb = t - rb * ncb;
      const int b = li & 1, s = li % nd;
      const int row = rb * FB_BM + r;
      const int col0 = cb * FB_BN + part * 8;  // < ncb * 32, within the padded scale arrays
      const int ea = row < rows ? eA[row] : 0;
      int fb[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) fb[u] = fB[col0 + u];
      ok = __all_sync(0xffffffffu, mbar_wait(acc_full(b), (li >> 1) & 1));
      if (!ok) break;
      tc_fence_after();
      // All seven level loads in flight at once, one wait.
      const uint32_t tbase = tmem + (uint32_t)(b * 256) + ((uint32_t)(q * 32) << 16) + (uint32_t)(part * 8);
      uint32_t v[FB_NLEV][8];
#pragma unroll
      for (int l = 0; l < FB_NLEV; ++l) tmem_ld8_nowait(tbase + (uint32_t)(l * FB_BN), v[l]);
      tmem_wait_ld();
      // the accumulator set is free once every warp has read it
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(acc_empty(b));
      // Levels in pairs: P = C_l * 2^7 + C_{l+1} is an exact int32;
      // Y = P23 2^28 + P45 2^14 + P67 + round(C8 / 2^7).
      long long Y[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        auto C = [&](int l) { return fbits(__uint_as_float(v[l][u])) - kMagicBits; };
        Y[u] = ((long long)(C(0) * 128 + C(1)) << 28) + ((long long)(C(2) * 128 + C(3)) << 14) +
               (long long)(C(4) * 128 + C(5)) + (long long)((C(6) + 64) >> 7);
      }
      ok = __all_sync(0xffffffffu, mbar_wait(d_full(s), (li / nd) & 1));
      if (!ok) break;
      // Rows and columns past M hold the TMA's zero fill and Y = 0 there;
      // the store clips them.
      const int E0 = ea - FB_B * (FB_LMAX - 1);
      unsigned char *slot = base + rowoff + (size_t)s * FB_DTILE;
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        double2 *p = reinterpret_cast<double2 *>(slot + 16 * ((c0 + u) ^ (r & 7)));
        double2 x = *p;
        x.x -= i64_scaled(Y[2 * u], E0 + fb[2 * u]);
        x.y -= i64_scaled(Y[2 * u + 1], E0 + fb[2 * u + 1]);
        *p = x;
      }
      fence_proxy_async_smem();
      __syncwarp();
      if (lane == 0) mbar_arrive(d_done(s));
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

// 2-D tensor map over M as row-major doubles: cols x rows, row pitch ldd
// doubles, 16 x 128 boxes, 128-byte swizzle (zero fill outside M).
cudaError_t make_map_f64(CUtensorMap *m, const double *base, long rows, long cols, long ldd) {
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

size_t f64tc_op_cols() { return (size_t)FB_MAX_ATOMS * 64; }

size_t f64tc_b_cols() { return 64; }

long f64tc_b_rows(long n) { return (2 * (n + 1) + FB_BN - 1) / FB_BN * FB_BROWS; }

cudaError_t launch_f64tc_update(Handle *h, int f, int k, double2 *M, const double2 *A, const double2 *W) {
  const long n = h->n, rows = n + h->E;
  const long cols = 2 * (n + 1);
  if (k < 1 || k > f64tc_max_k()) return cudaErrorInvalidValue;
  const int k2p = (2 * k + 15) / 16 * 16;
  const int kop = (FB_S * k2p + 63) / 64 * 64;
  const int natoms = kop / 64;
  const long ldk = (long)f64tc_op_cols();
  Lane &L = lane_of(h, f);
  cudaStream_t st = lane_stream(h, f);
  // operand rows have pitch ldk; each update fills its rows up to the pitch
  k_slice_A<<<(unsigned)((rows + 3) / 4), 128, 0, st>>>(A, rows, rows, k, k2p, (int)ldk,
                                                        static_cast<__nv_bfloat16 *>(L.A16), L.eA);
  k_slice_B<<<(unsigned)((cols + 3) / 4), 128, 0, st>>>(W, h->ldm, cols, k, static_cast<__nv_bfloat16 *>(L.B16),
                                                        L.fB);
  CUtensorMap ma, mb, md;
  cudaError_t e;
  if ((e = make_map_bf16(&ma, L.A16, h->a16_rows, kop, ldk, FB_BM)) != cudaSuccess) return e;
  if ((e = make_map_bf16(&mb, L.B16, h->b16_rows, 64, (long)f64tc_b_cols(), FB_BROWS)) != cudaSuccess) return e;
  if ((e = make_map_f64(&md, reinterpret_cast<const double *>(M), rows, cols, 2 * h->ldm)) != cudaSuccess) return e;
  if (g_num_sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&g_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (g_num_sms <= 0) g_num_sms = 1;
  }
  // two staged tiles of M when shared memory allows (k <= 24), else one
  const int nd = fb_smem(natoms, 2) <= (size_t)g_smem_optin ? 2 : 1;
  const size_t smem = fb_smem(natoms, nd);
  if (smem > (size_t)g_smem_optin) return cudaErrorInvalidValue;
  if ((e = cudaFuncSetAttribute(k_tc_update_f64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
      cudaSuccess)
    return e;
  const int nrb = (int)((rows + FB_BM - 1) / FB_BM), ncb = (int)((cols + FB_BN - 1) / FB_BN);
  const int ntiles = nrb * ncb;
  const int grid = ntiles < g_num_sms ? ntiles : g_num_sms;
  cudaEvent_t t0 = timing_mark(h, st);
  k_tc_update_f64<<<grid, FB_THREADS, smem, st>>>(ma, mb, md, (int)rows, (int)cols, ncb, ntiles, natoms, k2p, nd,
                                                  L.eA, L.fB, h->d_tc_err);
  const double cells = (double)rows * (double)(n + 1);
  timing_close(h, t0, T_UPDATE, 8.0 * k * cells, 2.0 * 16.0 * cells + 2.0 * kop * ((double)rows + (double)cols),
               0.0, st);
  h->nlaunch += 3;
  return cudaGetLastError();
}

}  // namespace pngf
