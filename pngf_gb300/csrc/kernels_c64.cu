// Complex64 form of the accept step: T is stored in complex64 and its rank-k
// update T -= A W runs on the 5th-generation tensor cores (tcgen05, sm_103a).
//
// Complex to real: with T viewed as a real matrix of 2N interleaved (re, im)
// columns, T_real -= A_real B_real^T where A_real[i, 2r..2r+1] = (Re, Im) of
// A[i, r] and, for output column 2j (real part) B_real[2j, 2r..2r+1] =
// (Re W[r,j], -Im W[r,j]) and for 2j+1 (imaginary part) (Im W[r,j], Re W[r,j]).
// Precision: 3xTF32 split products (x = hi + lo with hi, lo TF32), laid out
// along K as [A_hi | A_hi | A_lo] . [B_hi | B_lo | B_hi], so a single GEMM with
// K = 6k accumulates hi*hi + hi*lo + lo*hi in FP32 (TMEM). The small parts of
// the state that feed the objective (y, R, Eobj) are updated in FP64.
//
// Kernel k_tc_update (persistent, one CTA per SM, described at the kernel):
// TMA-staged tiles of T, an operand ring for A_op / B_op, two TMEM
// accumulators, eight epilogue warps and a TMA-store warp. Every mbarrier
// wait is bounded; on timeout the kernel records an error code, drains its own
// TMA copies, frees its TMEM and returns.
//
// Deferred updates: an accept appends its T part to pending factors U, Vt
// (k_defer_append) and the pending product is flushed by the same kernel with
// K = 6 x the pending rank (k_build_Aop_f / k_build_Bop_f build its operands).
//
// Drift check kernels (k_rows_*) and the FP64 <-> complex64 state conversion
// (k_split_M, k_merge_M) are here too.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cstdint>
#include <mutex>

#include "pngf_internal.h"
#include "tc_common.cuh"

namespace pngf {

namespace {

constexpr int TC_BM = 128;       // rows per tile (MMA M)
constexpr int TC_BK = 32;        // fp32 K elements per stage = one 128-byte swizzle row
constexpr uint32_t A_BYTES = TC_BM * TC_BK * 4;
constexpr uint32_t TC_DBOX = TC_BM * 128;  // 128 rows x 32 floats of T (one TMA box)
constexpr int TC_EPI_WARPS = 8;
constexpr int kLongKStages = 24;  // K stages per tile (rank >= 128) from which one staged tile of T is used
constexpr int TC_THREADS = 96 + 32 * TC_EPI_WARPS;  // producer, MMA and store warps + epilogue
using namespace tc;

// Shapes per output tile width BN (fp32 columns = the MMA N; 64 or 128,
// picked by the autotuner): operand stages in flight and shared memory.
// ND staged tiles of T (2: the next tile's T loads during this tile's
// epilogue; 1: for long K, where the MMAs of a tile outlast a T load and the
// shared memory serves a deeper operand ring instead). The operand ring takes
// what is left of the 227 KB: 3 or 6 stages with two tiles of T, 5 or 8 with one.
constexpr size_t kTcSmemOptin = 232448;
template <int BN, int ND> struct C64Tile {
  static constexpr uint32_t B_BYTES = BN * TC_BK * 4;  // one K stage of B
  static constexpr uint32_t STAGE = A_BYTES + B_BYTES;
  static constexpr uint32_t DTILE = (BN / 32) * TC_DBOX;  // a 128 x BN tile of T
  static constexpr int ST = (int)((kTcSmemOptin - 1024 - 256 - (size_t)ND * DTILE) / STAGE);  // operand stages
  static constexpr size_t SMEM = 1024 + ST * STAGE + ND * DTILE + 256;
  static_assert(ND == 1 || ND == 2, "one or two staged tiles of T");
  static_assert(SMEM <= kTcSmemOptin && (2 * ST + 10) * 8 + 4 <= 256, "shared memory and barrier block");
  // Instruction descriptor, kind::tf32: D f32 (bits 4-5 = 1), A and B tf32
  // (bits 7-9 and 10-12 = 2), both K-major (bits 15, 16 = 0), N >> 3 at bits
  // 17-22, M >> 4 at bits 24-28.
  static constexpr uint32_t IDESC =
      (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(TC_BM >> 4) << 24);
};

// T[i, j] -= sum_k Aop[i, k] Bop[j, k] for i < rows, j < cols (fp32 view of
// the complex64 T, reached through the tensor map tmD: 32 x 128 boxes,
// 128-byte swizzle). Aop / Bop come through TMA maps (K-major, 128-byte
// swizzle); nkb = K / 32.
//
// Persistent: one CTA per SM walks a contiguous range of 128 x BN tiles
// (row-block major). Warp 0 issues TMA loads: each tile of T into one of two
// shared-memory slots ahead of its epilogue, and the K stages of A and B
// into an ST-deep ring. Warp 1 allocates TMEM and issues the
// tcgen05.mma.kind::tf32 (M=128, N=BN, K=8) chains into one of two
// accumulators. Eight epilogue warps (two per TMEM lane quadrant, half the
// columns each) read the accumulator with tcgen05.ld and update the staged
// tile in place (thread = row; the swizzle makes these accesses conflict-free);
// warp 2 writes each finished tile back with a TMA store and frees its slot.
template <int BN, int ND>
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_tc_update(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                const __grid_constant__ CUtensorMap tmD, int cols, int ncb, int ntiles, int nkb, int *err) {
  using S = C64Tile<BN, ND>;
  constexpr int ST = S::ST;
  extern __shared__ unsigned char smem_raw[];
  unsigned char *base = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                          ~static_cast<uintptr_t>(1023));
  const uint32_t sbase = smem_u32(base);
  constexpr uint32_t dbase = ST * S::STAGE;  // byte offset of slot 0 from base
  const uint32_t sD0 = sbase + dbase;
  uint64_t *bars = reinterpret_cast<uint64_t *>(base + dbase + ND * S::DTILE);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(bars + 2 * ST + 10);
  const uint32_t bar0 = smem_u32(bars);
  auto full = [&](int s) { return bar0 + 8 * s; };
  auto empty = [&](int s) { return bar0 + 8 * (ST + s); };
  auto acc_full = [&](int b) { return bar0 + 8 * (2 * ST + b); };
  auto acc_empty = [&](int b) { return bar0 + 8 * (2 * ST + 2 + b); };
  auto d_full = [&](int s) { return bar0 + 8 * (2 * ST + 4 + s); };   // tile of T landed in slot s
  auto d_done = [&](int s) { return bar0 + 8 * (2 * ST + 6 + s); };   // epilogue finished slot s
  auto d_empty = [&](int s) { return bar0 + 8 * (2 * ST + 8 + s); };  // store has read slot s
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int t_begin = (int)(((long long)ntiles * blockIdx.x) / gridDim.x);
  const int t_end = (int)(((long long)ntiles * (blockIdx.x + 1)) / gridDim.x);

  if (threadIdx.x == 0) {
    for (int s = 0; s < ST; ++s) {
      mbar_init(full(s), 1);
      mbar_init(empty(s), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(acc_full(b), 1);
      mbar_init(acc_empty(b), TC_EPI_WARPS);
      mbar_init(d_full(b), 1);
      mbar_init(d_done(b), TC_EPI_WARPS);
      mbar_init(d_empty(b), 1);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) tmem_alloc(smem_u32(tslot), 2 * BN);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;

  if (warp == 0) {
    if (lane == 0) {
      bool ok = true;
      int g = 0, issuedD = 0;
      for (int t = t_begin; t < t_end && ok; ++t) {
        const int li = t - t_begin, rb = t / ncb, cb = t - rb * ncb;
        const int m0 = rb * TC_BM, n0 = cb * BN, s = li % ND;
        if (li >= ND && !mbar_wait(d_empty(s), ((li / ND) - 1) & 1)) { ok = false; break; }
        mbar_expect_tx(d_full(s), S::DTILE);
        for (int j = 0; j < BN / 32; ++j) tma_load_2d(sD0 + s * S::DTILE + j * TC_DBOX, &tmD, n0 + 32 * j, m0, d_full(s));
        ++issuedD;
        for (int kb = 0; kb < nkb; ++kb, ++g) {
          const int st = g % ST;
          if (g >= ST && !mbar_wait(empty(st), ((g / ST) - 1) & 1)) { ok = false; break; }
          mbar_expect_tx(full(st), S::STAGE);
          tma_load_2d(sbase + st * S::STAGE, &tmA, kb * TC_BK, m0, full(st));
          tma_load_2d(sbase + st * S::STAGE + A_BYTES, &tmB, kb * TC_BK, n0, full(st));
        }
      }
      if (!ok) atomicExch(err, 31);
      // Drain: every copy this thread issued has landed before the CTA exits.
      for (int q = g > ST ? g - ST : 0; q < g; ++q)
        if (!mbar_wait(full(q % ST), (q / ST) & 1)) atomicExch(err, 34);
      for (int q = issuedD > ND ? issuedD - ND : 0; q < issuedD; ++q)
        if (!mbar_wait(d_full(q % ND), (q / ND) & 1)) atomicExch(err, 34);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      bool ok = true;
      int g = 0;
      for (int t = t_begin; t < t_end && ok; ++t) {
        const int li = t - t_begin, b = li & 1;
        if (li >= 2 && !mbar_wait(acc_empty(b), ((li >> 1) - 1) & 1)) { ok = false; break; }
        tc_fence_after();
        const uint32_t acc = tmem + (uint32_t)(b * BN);
        for (int kb = 0; kb < nkb; ++kb, ++g) {
          const int st = g % ST;
          if (!mbar_wait(full(st), (g / ST) & 1)) { ok = false; break; }
          tc_fence_after();
          const uint64_t ad = sw128_desc(sbase + st * S::STAGE);
          const uint64_t bd = sw128_desc(sbase + st * S::STAGE + A_BYTES);
#pragma unroll
          for (int kk = 0; kk < TC_BK / 8; ++kk)  // K = 8 tf32 = 32 bytes per MMA: +2 in 16-byte units
            mma_tf32(acc, ad + 2 * kk, bd + 2 * kk, S::IDESC, (kb | kk) != 0);
          mma_commit(empty(st));
        }
        if (ok) mma_commit(acc_full(b));
      }
      if (!ok) atomicExch(err, 32);
    }
    __syncwarp();
  } else if (warp == 2) {
    if (lane == 0) {
      bool ok = true;
      for (int t = t_begin; t < t_end; ++t) {
        const int li = t - t_begin, rb = t / ncb, cb = t - rb * ncb, s = li % ND;
        if (!mbar_wait(d_done(s), (li / ND) & 1)) { ok = false; break; }
        for (int j = 0; j < BN / 32; ++j)  // rows / columns past T are clipped
          if (cb * BN + 32 * j < cols) tma_store_2d(&tmD, sD0 + s * S::DTILE + j * TC_DBOX, cb * BN + 32 * j, rb * TC_BM);
        bulk_commit();
        bulk_wait_read_all();
        mbar_arrive(d_empty(s));
      }
      bulk_wait_all();
      if (!ok) atomicExch(err, 35);
    }
    __syncwarp();
  } else {
    constexpr int HALF = BN / 2;      // columns per epilogue warp
    const int ew = warp - 3, part = ew >> 2, q = warp & 3;
    const int r = q * 32 + lane;      // row of the tile (TMEM lane)
    bool ok = true;
    for (int t = t_begin; t < t_end; ++t) {
      const int li = t - t_begin, b = li & 1, s = li % ND;
      ok = __all_sync(0xffffffffu, mbar_wait(acc_full(b), (li >> 1) & 1));
      if (!ok) break;
      tc_fence_after();
      uint32_t v[HALF];
      const uint32_t tbase = tmem + (uint32_t)(b * BN) + ((uint32_t)(q * 32) << 16) + (uint32_t)(part * HALF);
#pragma unroll
      for (int c = 0; c < HALF / 8; ++c) tmem_ld8_nowait(tbase + (uint32_t)(c * 8), v + 8 * c);
      tmem_wait_ld();
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(acc_empty(b));  // the accumulator may be refilled
      ok = __all_sync(0xffffffffu, mbar_wait(d_full(s), (li / ND) & 1));
      if (!ok) break;
      // Rows and columns past T hold the TMA's zero fill and a zero
      // accumulator; the store clips them.
      unsigned char *slot = base + dbase + (size_t)s * S::DTILE + (size_t)r * 128;
#pragma unroll
      for (int c4 = 0; c4 < HALF / 4; ++c4) {  // 16-byte chunks of this thread's columns
        const int col = part * HALF + 4 * c4;
        float4 *p = reinterpret_cast<float4 *>(slot + (col >> 5) * TC_DBOX + 16 * (((col & 31) >> 2) ^ (r & 7)));
        float4 x = *p;
        x.x -= __uint_as_float(v[4 * c4]);
        x.y -= __uint_as_float(v[4 * c4 + 1]);
        x.z -= __uint_as_float(v[4 * c4 + 2]);
        x.w -= __uint_as_float(v[4 * c4 + 3]);
        *p = x;
      }
      fence_proxy_async_smem();
      __syncwarp();
      if (lane == 0) mbar_arrive(d_done(s));
    }
    if (!ok && lane == 0) atomicExch(err, 33);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, 2 * BN);
  }
}

// ---------------------------------------------------------------------------
// Long-K form of the complex64 update (deferred flushes, build chunks):
// T -= A_real B_real^T with the 3xTF32 products taken from separate hi and lo
// operands -- per K stage the MMAs A_hi.B_hi, A_hi.B_lo and A_lo.B_hi -- so
// that each operand element crosses L2 once per tile instead of being stored
// and read twice as in the [A_hi | A_hi | A_lo] layout (a third less operand
// traffic), and with 128 x 256 output tiles (two TMEM accumulators of 256
// columns) so that each operand byte feeds twice the MMA work of a 128 x 128
// tile. At a flush's rank (K = 2r = 384 real columns at r = 192) the
// operands are re-read from L2 for every tile, which sets the pace; the T tile
// itself never enters shared memory: the epilogue writes -acc in 128 x 32
// boxes and the TMA unit adds them into T in L2 (cp.reduce.async.bulk.tensor
// .add), so T is read and written once in HBM and no staging slot waits on a
// load of T.
//
// Warp 0 issues the TMA loads of the K stages (hi parts and lo parts on their
// own full barriers, so that A_hi.B_hi starts while the lo parts land), warp
// 1 allocates TMEM and issues the MMAs, warps 2-9 are the epilogue in two
// groups of four (one warp per TMEM lane quarter), each group with one 16 KB
// staging box: a group reads 32 accumulator columns, writes them negated into
// its box, and its issuing thread adds the box into T; the groups alternate
// over the eight 32-column chunks of a tile. Every wait is bounded; on a
// timeout the kernel records an error code, drains its copies and reduces,
// frees its TMEM and returns.
//
// The CTAs take tiles in turn (tile blockIdx.x + i * gridDim.x in step i) in
// a column-major raster over bands of LK_GROUP row blocks, so that the tiles
// in flight at one time share one or two B panels and at most LK_GROUP A
// panels: the operands stay in L2 while T streams through it.
constexpr int LK_GROUP = 64;                           // row blocks per band of the raster
constexpr int LK_BN = 256;                             // fp32 output columns per tile (MMA N)
constexpr uint32_t LK_A = TC_BM * TC_BK * 4;           // one K stage of A_hi or A_lo (16 KB)
constexpr uint32_t LK_B = LK_BN * TC_BK * 4;           // one K stage of B_hi or B_lo (32 KB)
constexpr uint32_t LK_HALF = LK_A + LK_B;              // hi (or lo) part of a stage
constexpr uint32_t LK_STAGE = 2 * LK_HALF;             // 96 KB
constexpr int LK_ST = 2;                               // stages in the ring
constexpr uint32_t LK_STG = TC_BM * 128;               // a 128 x 32-float box of the epilogue output
constexpr int LK_EPI_WARPS = 8;                        // two groups of four
constexpr int LK_CHUNKS = LK_BN / 32;                  // 32-column chunks per tile
constexpr int LK_THREADS = 64 + 32 * LK_EPI_WARPS;     // producer, MMA, epilogue
constexpr int LK_NBARS = 3 * LK_ST + 8;                // full_hi, full_lo, empty; acc_full/empty; stg_full/free
constexpr size_t LK_SMEM = 1024 + (size_t)LK_ST * LK_STAGE + 2 * LK_STG + 256;
static_assert(LK_SMEM <= kTcSmemOptin && LK_NBARS * 8 + 4 <= 256, "long-K shared memory and barrier block");
constexpr uint32_t LK_IDESC =
    (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(LK_BN >> 3) << 17) | ((uint32_t)(TC_BM >> 4) << 24);

// Row and column block of tile t in the banded column-major raster.
__device__ __forceinline__ void lk_tile(int t, int nrb, int ncb, int &rb, int &cb) {
  const int per = LK_GROUP * ncb, band = t / per, first = band * LK_GROUP, w = t - band * per;
  const int rows = min(nrb - first, LK_GROUP);
  rb = first + w % rows;
  cb = w / rows;
}

__global__ void __launch_bounds__(LK_THREADS, 1)
    k_tc_update_longk(const __grid_constant__ CUtensorMap tmAhi, const __grid_constant__ CUtensorMap tmAlo,
                      const __grid_constant__ CUtensorMap tmBhi, const __grid_constant__ CUtensorMap tmBlo,
                      const __grid_constant__ CUtensorMap tmD, int cols, int ncb, int ntiles, int nkb, int *err) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char *base = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                          ~static_cast<uintptr_t>(1023));
  const uint32_t sbase = smem_u32(base);
  constexpr uint32_t stg_off = LK_ST * LK_STAGE;  // staging boxes after the ring (1024-aligned)
  uint64_t *bars = reinterpret_cast<uint64_t *>(base + stg_off + 2 * LK_STG);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(bars + LK_NBARS);
  const uint32_t bar0 = smem_u32(bars);
  auto full_hi = [&](int s) { return bar0 + 8u * (uint32_t)s; };
  auto full_lo = [&](int s) { return bar0 + 8u * (uint32_t)(LK_ST + s); };
  auto empty = [&](int s) { return bar0 + 8u * (uint32_t)(2 * LK_ST + s); };
  auto acc_full = [&](int b) { return bar0 + 8u * (uint32_t)(3 * LK_ST + b); };
  auto acc_empty = [&](int b) { return bar0 + 8u * (uint32_t)(3 * LK_ST + 2 + b); };
  auto stg_full = [&](int g) { return bar0 + 8u * (uint32_t)(3 * LK_ST + 4 + g); };
  auto stg_free = [&](int g) { return bar0 + 8u * (uint32_t)(3 * LK_ST + 6 + g); };
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nrb = ntiles / ncb;
  // this CTA's tiles: t = blockIdx.x + li * gridDim.x for li < nloc
  const int nloc = (int)blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;

  if (threadIdx.x == 0) {
    for (int s = 0; s < LK_ST; ++s) {
      mbar_init(full_hi(s), 1);
      mbar_init(full_lo(s), 1);
      mbar_init(empty(s), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(acc_full(b), 1);
      mbar_init(acc_empty(b), LK_EPI_WARPS);
      mbar_init(stg_full(b), 4);
      mbar_init(stg_free(b), 1);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) tmem_alloc(smem_u32(tslot), 2 * LK_BN);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;

  if (warp == 0) {
    if (lane == 0) {
      bool ok = true;
      int g = 0;
      for (int li = 0; li < nloc && ok; ++li) {
        int rb, cb;
        lk_tile((int)blockIdx.x + li * (int)gridDim.x, nrb, ncb, rb, cb);
        const int m0 = rb * TC_BM, n0 = cb * LK_BN;
        for (int kb = 0; kb < nkb; ++kb, ++g) {
          const int st = g % LK_ST;
          if (g >= LK_ST && !mbar_wait(empty(st), ((g / LK_ST) - 1) & 1)) { ok = false; break; }
          const uint32_t sa = sbase + (uint32_t)st * LK_STAGE;
          mbar_expect_tx(full_hi(st), LK_HALF);
          tma_load_2d(sa, &tmAhi, kb * TC_BK, m0, full_hi(st));
          tma_load_2d(sa + LK_A, &tmBhi, kb * TC_BK, n0, full_hi(st));
          mbar_expect_tx(full_lo(st), LK_HALF);
          tma_load_2d(sa + LK_HALF, &tmAlo, kb * TC_BK, m0, full_lo(st));
          tma_load_2d(sa + LK_HALF + LK_A, &tmBlo, kb * TC_BK, n0, full_lo(st));
        }
      }
      if (!ok) atomicExch(err, 41);
      // Drain: every stage issued has landed before the CTA can exit.
      for (int q = g > LK_ST ? g - LK_ST : 0; q < g; ++q) {
        if (!mbar_wait(full_hi(q % LK_ST), (q / LK_ST) & 1)) atomicExch(err, 44);
        if (!mbar_wait(full_lo(q % LK_ST), (q / LK_ST) & 1)) atomicExch(err, 44);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      bool ok = true;
      int g = 0;
      for (int li = 0; li < nloc && ok; ++li) {
        const int b = li & 1;
        if (li >= 2 && !mbar_wait(acc_empty(b), ((li >> 1) - 1) & 1)) { ok = false; break; }
        tc_fence_after();
        const uint32_t acc = tmem + (uint32_t)(b * LK_BN);
        for (int kb = 0; kb < nkb; ++kb, ++g) {
          const int st = g % LK_ST;
          const uint32_t sa = sbase + (uint32_t)st * LK_STAGE;
          const uint64_t ahi = sw128_desc(sa), bhi = sw128_desc(sa + LK_A);
          const uint64_t alo = sw128_desc(sa + LK_HALF), blo = sw128_desc(sa + LK_HALF + LK_A);
          if (!mbar_wait(full_hi(st), (g / LK_ST) & 1)) { ok = false; break; }
          tc_fence_after();
#pragma unroll
          for (int kk = 0; kk < TC_BK / 8; ++kk)  // K = 8 tf32 = 32 bytes per MMA: +2 in 16-byte units
            mma_tf32(acc, ahi + 2 * kk, bhi + 2 * kk, LK_IDESC, (kb | kk) != 0);
          if (!mbar_wait(full_lo(st), (g / LK_ST) & 1)) { ok = false; break; }
          tc_fence_after();
#pragma unroll
          for (int kk = 0; kk < TC_BK / 8; ++kk) {
            mma_tf32(acc, ahi + 2 * kk, blo + 2 * kk, LK_IDESC, 1u);
            mma_tf32(acc, alo + 2 * kk, bhi + 2 * kk, LK_IDESC, 1u);
          }
          mma_commit(empty(st));
        }
        if (ok) mma_commit(acc_full(b));
      }
      if (!ok) atomicExch(err, 42);
    }
    __syncwarp();
  } else {
    const int ew = warp - 2;          // 0..7
    const int grp = ew >> 2;          // group 0: warps 2-5, group 1: warps 6-9
    const int q = warp & 3;           // TMEM lanes 32q .. 32q+31 (each group covers all four)
    const int r = q * 32 + lane;      // row of the tile
    const bool issuer = (q == 0) && lane == 0;  // one thread per group issues its reductions
    const uint32_t stg = sbase + stg_off + (uint32_t)grp * LK_STG;
    unsigned char *stg_row = base + stg_off + (size_t)grp * LK_STG + (size_t)r * 128;
    bool ok = true;
    int n = 0;  // chunks this group has written (its staging box's uses)
    for (int li = 0; li < nloc && ok; ++li) {
      const int b = li & 1;
      int rb, cb;
      lk_tile((int)blockIdx.x + li * (int)gridDim.x, nrb, ncb, rb, cb);
      ok = __all_sync(0xffffffffu, mbar_wait(acc_full(b), (li >> 1) & 1));
      if (!ok) break;
      tc_fence_after();
      for (int c = grp; c < LK_CHUNKS; c += 2, ++n) {
        uint32_t v[32];
        const uint32_t ta = tmem + (uint32_t)(b * LK_BN + c * 32) + ((uint32_t)(q * 32) << 16);
#pragma unroll
        for (int u = 0; u < 4; ++u) tmem_ld8_nowait(ta + (uint32_t)(8 * u), v + 8 * u);
        tmem_wait_ld();
        if (c + 2 >= LK_CHUNKS) {  // this warp's last read of the accumulator
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(acc_empty(b));
        }
        // the box is free once the group's previous reduction has read it
        if (n > 0) {
          ok = __all_sync(0xffffffffu, mbar_wait(stg_free(grp), (n - 1) & 1));
          if (!ok) break;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {  // 16-byte unit u of the row, 128-byte swizzle
          float4 x;
          x.x = -__uint_as_float(v[4 * u]);
          x.y = -__uint_as_float(v[4 * u + 1]);
          x.z = -__uint_as_float(v[4 * u + 2]);
          x.w = -__uint_as_float(v[4 * u + 3]);
          *reinterpret_cast<float4 *>(stg_row + 16 * (u ^ (r & 7))) = x;
        }
        fence_proxy_async_smem();
        __syncwarp();
        if (lane == 0) mbar_arrive(stg_full(grp));
        if (issuer) {
          if (!mbar_wait(stg_full(grp), n & 1)) {
            ok = false;
          } else {
            const int x0 = cb * LK_BN + 32 * c;
            if (x0 < cols) tma_reduce_add_2d(&tmD, stg, x0, rb * TC_BM);  // rows past T are clipped
            bulk_commit();
            bulk_wait_read_all();
            mbar_arrive(stg_free(grp));
          }
        }
        ok = __all_sync(0xffffffffu, ok);
        if (!ok) break;
      }
    }
    if (issuer) bulk_wait_all();  // every reduction of this group has completed
    if (!ok && lane == 0) atomicExch(err, 43);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, 2 * LK_BN);
  }
}

// A_op rows i < n: 3xTF32 segments of the interleaved real form of A[i, :].
// One block per 32 rows: A's 32 x k block is read column-coalesced into shared
// memory, then the rows of A_op are written along K.
constexpr int BO_ROWS = 32;   // A_op rows per block
constexpr int BO_COLS = 16;   // complex columns of W per block (32 rows of B_op)
__global__ void __launch_bounds__(256) k_build_Aop(const double2 *__restrict__ A, long lda, long n, int k, int Kt,
                                                   long ldk, float *__restrict__ Aop) {
  extern __shared__ double2 bsm[];  // k x (BO_ROWS + 1)
  const long i0 = (long)blockIdx.x * BO_ROWS;
  for (int idx = threadIdx.x; idx < k * BO_ROWS; idx += blockDim.x) {
    const int r = idx / BO_ROWS, ii = idx - r * BO_ROWS;
    bsm[r * (BO_ROWS + 1) + ii] = i0 + ii < n ? A[(size_t)r * lda + i0 + ii] : make_double2(0.0, 0.0);
  }
  __syncthreads();
  const int k2 = 2 * k;
  for (int idx = threadIdx.x; idx < BO_ROWS * Kt; idx += blockDim.x) {
    const int ii = idx / Kt, c = idx - ii * Kt;
    const long i = i0 + ii;
    if (i >= n) break;
    float v = 0.f;
    if (c < 3 * k2) {
      const int seg = c / k2, w = c - seg * k2, r = w >> 1;
      const double2 a = bsm[r * (BO_ROWS + 1) + ii];
      const float x = (float)((w & 1) ? a.y : a.x);
      const float hi = to_tf32(x);
      v = seg == 2 ? to_tf32(x - hi) : hi;
    }
    Aop[(size_t)i * ldk + c] = v;
  }
}

// B_op rows j' < 2n: output column j' = 2j (real part) or 2j+1 (imaginary).
// One block per 16 columns of W (32 rows of B_op), staged like k_build_Aop.
__global__ void __launch_bounds__(256) k_build_Bop(const double2 *__restrict__ W, long ldw, long n, int k, int Kt,
                                                   long ldk, float *__restrict__ Bop) {
  extern __shared__ double2 bsm[];  // k x (BO_COLS + 1)
  const long j0 = (long)blockIdx.x * BO_COLS;
  for (int idx = threadIdx.x; idx < k * BO_COLS; idx += blockDim.x) {
    const int r = idx / BO_COLS, jj = idx - r * BO_COLS;
    bsm[r * (BO_COLS + 1) + jj] = j0 + jj < n ? W[(size_t)r * ldw + j0 + jj] : make_double2(0.0, 0.0);
  }
  __syncthreads();
  const int k2 = 2 * k;
  for (int idx = threadIdx.x; idx < 2 * BO_COLS * Kt; idx += blockDim.x) {
    const int jl = idx / Kt, c = idx - jl * Kt;
    const long jp = 2 * j0 + jl;
    if (jp >= 2 * n) break;
    float v = 0.f;
    if (c < 3 * k2) {
      const int seg = c / k2, w = c - seg * k2, r = w >> 1;
      const double2 wv = bsm[r * (BO_COLS + 1) + (jl >> 1)];
      double b;
      if ((jp & 1) == 0) b = (w & 1) ? -wv.y : wv.x;  // Re out: Re A Re W - Im A Im W
      else b = (w & 1) ? wv.x : wv.y;                 // Im out: Re A Im W + Im A Re W
      const float x = (float)b;
      const float hi = to_tf32(x);
      v = seg == 1 ? to_tf32(x - hi) : hi;
    }
    Bop[(size_t)jp * ldk + c] = v;
  }
}

// Deferred updates: appends the T part of an accept to the pending factors,
// U[i][rp + c] = A[i][c] and Vt[j][rp + c] = W[c][j] (i, j < N), in complex64.
// A CTA takes DA_ROWS rows: it reads A's and W's columns along the rows
// (coalesced) into shared memory and writes each row's k new entries as one
// contiguous run, threads along the run.
constexpr int DA_ROWS = 32;
__global__ void __launch_bounds__(256) k_defer_append(const double2 *__restrict__ A, long lda,
                                                      const double2 *__restrict__ W, long ldw, long n, int k,
                                                      int rp, int rcap, float2 *__restrict__ U,
                                                      float2 *__restrict__ Vt) {
  extern __shared__ float2 da[];  // [2][k][DA_ROWS + 1] (padded: a run's reads fall in different banks)
  constexpr int P = DA_ROWS + 1;
  float2 *sa = da, *sw = da + (size_t)k * P;
  const long i0 = (long)blockIdx.x * DA_ROWS;
  const int t = threadIdx.x;
  for (int idx = t; idx < k * DA_ROWS; idx += blockDim.x) {
    const int c = idx / DA_ROWS, r = idx % DA_ROWS;
    const long i = i0 + r;
    if (i < n) {
      const double2 a = A[(size_t)c * lda + i], w = W[(size_t)c * ldw + i];
      sa[c * P + r] = make_float2((float)a.x, (float)a.y);
      sw[c * P + r] = make_float2((float)w.x, (float)w.y);
    }
  }
  __syncthreads();
  for (int idx = t; idx < k * DA_ROWS; idx += blockDim.x) {
    const int r = idx / k, c = idx % k;
    const long i = i0 + r;
    if (i < n) {
      U[(size_t)i * rcap + rp + c] = sa[c * P + r];
      Vt[(size_t)i * rcap + rp + c] = sw[c * P + r];
    }
  }
}

// A_op and B_op (as k_build_Aop / k_build_Bop) from the pending factors:
// A = U (rows i, rank r), W[r][j] = Vt[j][r].
__global__ void k_build_Aop_f(const float2 *__restrict__ U, int rcap, long n, int k, int Kt, long ldk,
                              float *__restrict__ Aop) {
  const long i = (long)blockIdx.y;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || c >= Kt) return;
  float v = 0.f;
  const int k2 = 2 * k;
  if (c < 3 * k2) {
    const int seg = c / k2, w = c - seg * k2, r = w >> 1;
    const float2 a = U[(size_t)i * rcap + r];
    const float x = (w & 1) ? a.y : a.x;
    const float hi = to_tf32(x);
    v = seg == 2 ? to_tf32(x - hi) : hi;
  }
  Aop[(size_t)i * ldk + c] = v;
}

__global__ void k_build_Bop_f(const float2 *__restrict__ Vt, int rcap, long n, int k, int Kt, long ldk,
                              float *__restrict__ Bop) {
  const long jp = (long)blockIdx.y;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (jp >= 2 * n || c >= Kt) return;
  float v = 0.f;
  const int k2 = 2 * k;
  if (c < 3 * k2) {
    const int seg = c / k2, w = c - seg * k2, r = w >> 1;
    const float2 wv = Vt[(size_t)(jp >> 1) * rcap + r];
    float b;
    if ((jp & 1) == 0) b = (w & 1) ? -wv.y : wv.x;  // Re out: Re A Re W - Im A Im W
    else b = (w & 1) ? wv.x : wv.y;                 // Im out: Re A Im W + Im A Re W
    const float hi = to_tf32(b);
    v = seg == 1 ? to_tf32(b - hi) : hi;
  }
  Bop[(size_t)jp * ldk + c] = v;
}

// Operands of the long-K kernel: the interleaved real forms of A and B split
// into TF32 hi and lo parts, stored as separate matrices (rows x K2, K2 = 2k
// padded to 32, zeros past 2k): A_hi at Ahi, A_lo at Alo, B likewise. From
// the pending factors (A = U, W[r][j] = Vt[j][r]) ...
__global__ void k_build_hl_Af(const float2 *__restrict__ U, int rcap, long n, int k, int K2, float *__restrict__ Ahi,
                              float *__restrict__ Alo) {
  const long i = (long)blockIdx.y;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || c >= K2) return;
  float hi = 0.f, lo = 0.f;
  if (c < 2 * k) {
    const float2 a = U[(size_t)i * rcap + (c >> 1)];
    const float x = (c & 1) ? a.y : a.x;
    hi = to_tf32(x);
    lo = to_tf32(x - hi);
  }
  Ahi[(size_t)i * K2 + c] = hi;
  Alo[(size_t)i * K2 + c] = lo;
}

__global__ void k_build_hl_Bf(const float2 *__restrict__ Vt, int rcap, long n, int k, int K2, float *__restrict__ Bhi,
                              float *__restrict__ Blo) {
  const long jp = (long)blockIdx.y;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (jp >= 2 * n || c >= K2) return;
  float hi = 0.f, lo = 0.f;
  if (c < 2 * k) {
    const float2 wv = Vt[(size_t)(jp >> 1) * rcap + (c >> 1)];
    float b;
    if ((jp & 1) == 0) b = (c & 1) ? -wv.y : wv.x;  // Re out: Re A Re W - Im A Im W
    else b = (c & 1) ? wv.x : wv.y;                 // Im out: Re A Im W + Im A Re W
    hi = to_tf32(b);
    lo = to_tf32(b - hi);
  }
  Bhi[(size_t)jp * K2 + c] = hi;
  Blo[(size_t)jp * K2 + c] = lo;
}

// ... and from an accept's FP64 factors A ((n+E) x k, column-major, lda) and W
// (k x ldw row-major), rounded to FP32 first as k_build_Aop / k_build_Bop do,
// staged through shared memory like them (coalesced reads of A's columns and
// W's rows, rows of the operands written along K).
__global__ void __launch_bounds__(256) k_build_hl_A(const double2 *__restrict__ A, long lda, long n, int k, int K2,
                                                    float *__restrict__ Ahi, float *__restrict__ Alo) {
  extern __shared__ double2 bsm[];  // k x (BO_ROWS + 1)
  const long i0 = (long)blockIdx.x * BO_ROWS;
  for (int idx = threadIdx.x; idx < k * BO_ROWS; idx += blockDim.x) {
    const int r = idx / BO_ROWS, ii = idx - r * BO_ROWS;
    bsm[r * (BO_ROWS + 1) + ii] = i0 + ii < n ? A[(size_t)r * lda + i0 + ii] : make_double2(0.0, 0.0);
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < BO_ROWS * K2; idx += blockDim.x) {
    const int ii = idx / K2, c = idx - ii * K2;
    const long i = i0 + ii;
    if (i >= n) break;
    float hi = 0.f, lo = 0.f;
    if (c < 2 * k) {
      const double2 a = bsm[(c >> 1) * (BO_ROWS + 1) + ii];
      const float x = (float)((c & 1) ? a.y : a.x);
      hi = to_tf32(x);
      lo = to_tf32(x - hi);
    }
    Ahi[(size_t)i * K2 + c] = hi;
    Alo[(size_t)i * K2 + c] = lo;
  }
}

__global__ void __launch_bounds__(256) k_build_hl_B(const double2 *__restrict__ W, long ldw, long n, int k, int K2,
                                                    float *__restrict__ Bhi, float *__restrict__ Blo) {
  extern __shared__ double2 bsm[];  // k x (BO_COLS + 1)
  const long j0 = (long)blockIdx.x * BO_COLS;
  for (int idx = threadIdx.x; idx < k * BO_COLS; idx += blockDim.x) {
    const int r = idx / BO_COLS, jj = idx - r * BO_COLS;
    bsm[r * (BO_COLS + 1) + jj] = j0 + jj < n ? W[(size_t)r * ldw + j0 + jj] : make_double2(0.0, 0.0);
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < 2 * BO_COLS * K2; idx += blockDim.x) {
    const int jl = idx / K2, c = idx - jl * K2;
    const long jp = 2 * j0 + jl;
    if (jp >= 2 * n) break;
    float hi = 0.f, lo = 0.f;
    if (c < 2 * k) {
      const double2 wv = bsm[(c >> 1) * (BO_COLS + 1) + (jl >> 1)];
      double b;
      if ((jp & 1) == 0) b = (c & 1) ? -wv.y : wv.x;
      else b = (c & 1) ? wv.x : wv.y;
      const float x = (float)b;
      hi = to_tf32(x);
      lo = to_tf32(x - hi);
    }
    Bhi[(size_t)jp * K2 + c] = hi;
    Blo[(size_t)jp * K2 + c] = lo;
  }
}

// FP64 part of the complex64 accept: y_i -= sum_r A[i,r] W[r,N] (i < N) and
// R[e, j] -= sum_r A[N+e, r] W[r, j] (j <= N).
__global__ void k_c64_side_update(double2 *__restrict__ y64, double2 *__restrict__ R64, long n, int E, long ldm,
                                  const double2 *__restrict__ A, long lda, const double2 *__restrict__ W, int k) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) {
    double2 acc = make_double2(0.0, 0.0);
    for (int r = 0; r < k; ++r) {
      const double2 a = A[(size_t)r * lda + t], w = W[(size_t)r * ldm + n];
      acc.x += a.x * w.x - a.y * w.y;
      acc.y += a.x * w.y + a.y * w.x;
    }
    y64[t].x -= acc.x;
    y64[t].y -= acc.y;
    return;
  }
  const long u = t - n;
  if (u >= (long)E * (n + 1)) return;
  const int e = (int)(u / (n + 1));
  const long j = u - (long)e * (n + 1);
  double2 acc = make_double2(0.0, 0.0);
  for (int r = 0; r < k; ++r) {
    const double2 a = A[(size_t)r * lda + n + e], w = W[(size_t)r * ldm + j];
    acc.x += a.x * w.x - a.y * w.y;
    acc.y += a.x * w.y + a.y * w.x;
  }
  double2 *p = R64 + (size_t)e * ldm + j;
  p->x -= acc.x;
  p->y -= acc.y;
}

__global__ void k_split_M(const double2 *__restrict__ M, long n, int E, long ldm, float2 *__restrict__ T32,
                          double2 *__restrict__ y64, double2 *__restrict__ R64) {
  const long i = blockIdx.y;
  const long j = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= ldm) return;
  const double2 v = M[(size_t)i * ldm + j];
  if (i < n) {
    T32[(size_t)i * ldm + j] = j < n ? make_float2((float)v.x, (float)v.y) : make_float2(0.f, 0.f);
    if (j == n) y64[i] = v;
  } else {
    R64[(size_t)(i - n) * ldm + j] = v;
  }
}

__global__ void k_merge_M(const float2 *__restrict__ T32, const double2 *__restrict__ y64,
                          const double2 *__restrict__ R64, long n, int E, long ldm, double2 *__restrict__ M) {
  const long i = blockIdx.y;
  const long j = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= ldm) return;
  double2 v;
  if (i < n) {
    if (j < n) {
      const float2 t = T32[(size_t)i * ldm + j];
      v = make_double2(t.x, t.y);
    } else {
      v = j == n ? y64[i] : make_double2(0.0, 0.0);
    }
  } else {
    v = R64[(size_t)(i - n) * ldm + j];
  }
  M[(size_t)i * ldm + j] = v;
}

// ---------------------------------------------------------------------------
// FP64 drift check of the complex64 T on sampled rows.
//
// The exact rows satisfy X C = H_rows with C = I + P H, H = G - I. Starting
// from X = T32[rows], iterative refinement X <- X - (X C - H_rows) C^-1 uses
// the identity C^-1 = I - P T with the complex64 T as the approximate
// inverse. A sweep multiplies the error of X by about the relative error of
// that inverse (the drift d itself, plus complex64 rounding), so after one
// sweep X is within ~d^2 of the exact rows: the drift it measures is exact
// to ~d relative (d <= 1e-4 below any refresh threshold), and a second sweep
// would only sharpen digits the check does not report.

constexpr int DR_MAX_ROWS = 8;

// out[r][j] = sum_{l in P} X[r][P_l] H[P_l][j], one warp per column j (lanes
// walk P, so the reads of column j of G are contiguous). NR rows exactly, so
// that no FP64 instruction is issued for absent rows.
template <int NR>
__global__ void k_rows_PH(const double2 *__restrict__ X, long n, const int *__restrict__ Pidx, int np,
                          const double2 *__restrict__ G, double2 *__restrict__ out) {
  constexpr int nr = NR;
  const long j = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (j >= n) return;
  double2 acc[NR];
#pragma unroll
  for (int r = 0; r < NR; ++r) acc[r] = make_double2(0.0, 0.0);
  for (int q = lane; q < np; q += 32) {
    const int l = Pidx[q];
    double2 hv = G[(size_t)j * n + l];
    if (l == j) hv.x -= 1.0;
#pragma unroll
    for (int r = 0; r < NR; ++r) {
      const double2 x = X[(size_t)r * n + l];
      acc[r].x += x.x * hv.x - x.y * hv.y;
      acc[r].y += x.x * hv.y + x.y * hv.x;
    }
  }
#pragma unroll
  for (int r = 0; r < NR; ++r) {
    for (int o = 16; o; o >>= 1) {
      acc[r].x += __shfl_xor_sync(0xffffffffu, acc[r].x, o);
      acc[r].y += __shfl_xor_sync(0xffffffffu, acc[r].y, o);
    }
    if (lane == 0 && r < nr) out[(size_t)r * n + j] = acc[r];
  }
}

// Rk[r][j] = X[r][j] + PH[r][j] - H[rows_r][j].
__global__ void k_rows_residual(const double2 *__restrict__ X, const double2 *__restrict__ PH,
                                const double2 *__restrict__ G, const int *__restrict__ rows, int nr, long n,
                                double2 *__restrict__ Rk) {
  const long j = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  for (int r = 0; r < nr; ++r) {
    const long i = rows[r];
    double2 h = G[(size_t)j * n + i];
    if (i == j) h.x -= 1.0;
    const double2 x = X[(size_t)r * n + j], p = PH[(size_t)r * n + j];
    Rk[(size_t)r * n + j] = make_double2(x.x + p.x - h.x, x.y + p.y - h.y);
  }
}

// X[r][j] -= Rk[r][j] - sum_{l in P} Rk[r][P_l] T[P_l][j]: 32 columns per CTA
// (lane = column, so each warp reads 256 contiguous bytes of a row of T), the
// sum over P split across the CTA's 8 warps and reduced in shared memory.
template <int NR>
__global__ void __launch_bounds__(256) k_rows_refine(double2 *__restrict__ X, const double2 *__restrict__ Rk, long n,
                                                     const int *__restrict__ Pidx, int np,
                                                     const float2 *__restrict__ T32, long ldm) {
  constexpr int nr = NR;
  __shared__ double2 part[8][NR][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const long j = (long)blockIdx.x * 32 + lane;
  double2 acc[NR];
#pragma unroll
  for (int r = 0; r < NR; ++r) acc[r] = make_double2(0.0, 0.0);
  if (j < n)
    for (int q = w; q < np; q += 8) {
      const int l = Pidx[q];
      const float2 tf = T32[(size_t)l * ldm + j];
      const double2 t = make_double2(tf.x, tf.y);
#pragma unroll
      for (int r = 0; r < NR; ++r) {
        const double2 rv = Rk[(size_t)r * n + l];
        acc[r].x += rv.x * t.x - rv.y * t.y;
        acc[r].y += rv.x * t.y + rv.y * t.x;
      }
    }
#pragma unroll
  for (int r = 0; r < NR; ++r) part[w][r][lane] = acc[r];
  __syncthreads();
  if (w == 0 && j < n)
    for (int r = 0; r < nr; ++r) {
      double2 sum = part[0][r][lane];
      for (int u = 1; u < 8; ++u) {
        sum.x += part[u][r][lane].x;
        sum.y += part[u][r][lane].y;
      }
      const double2 rv = Rk[(size_t)r * n + j];
      double2 &x = X[(size_t)r * n + j];
      x.x -= rv.x - sum.x;
      x.y -= rv.y - sum.y;
    }
}

__global__ void k_rows_load(const float2 *__restrict__ T32, long ldm, const int *__restrict__ rows, int nr, long n,
                            double2 *__restrict__ X) {
  const long j = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  for (int r = 0; r < nr; ++r) {
    const float2 t = T32[(size_t)rows[r] * ldm + j];
    X[(size_t)r * n + j] = make_double2(t.x, t.y);
  }
}

// out[0] = max |T32[rows] - X|, out[1] = max |X| (non-negative doubles: their
// bit patterns order like unsigned integers).
__global__ void k_rows_compare(const float2 *__restrict__ T32, long ldm, const int *__restrict__ rows, int nr, long n,
                               const double2 *__restrict__ X, unsigned long long *out) {
  const long j = (long)blockIdx.x * blockDim.x + threadIdx.x;
  double dmax = 0.0, xmax = 0.0;
  if (j < n)
    for (int r = 0; r < nr; ++r) {
      const float2 t = T32[(size_t)rows[r] * ldm + j];
      const double2 x = X[(size_t)r * n + j];
      dmax = fmax(dmax, hypot(t.x - x.x, t.y - x.y));
      xmax = fmax(xmax, hypot(x.x, x.y));
    }
  for (int o = 16; o; o >>= 1) {
    dmax = fmax(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
    xmax = fmax(xmax, __shfl_xor_sync(0xffffffffu, xmax, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(out, (unsigned long long)__double_as_longlong(dmax));
    atomicMax(out + 1, (unsigned long long)__double_as_longlong(xmax));
  }
}

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
int g_c64_sms = 0;
std::once_flag g_encode_once;

cudaError_t get_encoder() {
  std::call_once(g_encode_once, [] {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  });
  return g_encode ? cudaSuccess : cudaErrorNotSupported;
}

// 2-D fp32 tensor map over rows x K (K contiguous, row pitch ldk floats),
// box 32 x box_rows, 128-byte swizzle.
cudaError_t make_map(CUtensorMap *m, const float *base, long rows, int K, long ldk, int box_rows) {
  const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)ldk * sizeof(float)};
  const cuuint32_t box[2] = {(cuuint32_t)TC_BK, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(base), dims, strides, box,
                              estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

}  // namespace

cudaError_t launch_split_M(Handle *h, int f) {
  Freq &q = h->f[f];
  dim3 g((unsigned)((h->ldm + 255) / 256), (unsigned)(h->n + h->E));
  k_split_M<<<g, 256, 0, lane_stream(h, f)>>>(q.M64, h->n, h->E, h->ldm, q.T32, q.y64, q.R64);
  h->nlaunch += 1;
  return cudaGetLastError();
}

cudaError_t launch_drift_rows(Handle *h, int f, const int *d_rows, int nr, const int *d_P, int np, double2 *X,
                              double2 *PH, double2 *Rk, unsigned long long *d_out) {
  Freq &q = h->f[f];
  const long n = h->n;
  if (nr < 1 || nr > DR_MAX_ROWS) return cudaErrorInvalidValue;
  const unsigned g1 = (unsigned)((n + 255) / 256), gw = (unsigned)((n * 32 + 255) / 256);
  k_rows_load<<<g1, 256, 0, h->stream>>>(q.T32, h->ldm, d_rows, nr, n, X);
  const unsigned gr = (unsigned)((n + 31) / 32);
  switch (nr) {
#define PNGF_DRIFT_ROWS(NRV)                                                                     \
  case NRV:                                                                                      \
    k_rows_PH<NRV><<<gw, 256, 0, h->stream>>>(X, n, d_P, np, q.G, PH);                           \
    k_rows_residual<<<g1, 256, 0, h->stream>>>(X, PH, q.G, d_rows, nr, n, Rk);                   \
    k_rows_refine<NRV><<<gr, 256, 0, h->stream>>>(X, Rk, n, d_P, np, q.T32, h->ldm);             \
    break;
    PNGF_DRIFT_ROWS(1)
    PNGF_DRIFT_ROWS(2)
    PNGF_DRIFT_ROWS(3)
    PNGF_DRIFT_ROWS(4)
    PNGF_DRIFT_ROWS(5)
    PNGF_DRIFT_ROWS(6)
    PNGF_DRIFT_ROWS(7)
    PNGF_DRIFT_ROWS(8)
#undef PNGF_DRIFT_ROWS
    default:
      return cudaErrorInvalidValue;
  }
  k_rows_compare<<<g1, 256, 0, h->stream>>>(q.T32, h->ldm, d_rows, nr, n, X, d_out);
  h->nlaunch += 5;
  return cudaGetLastError();
}

cudaError_t launch_merge_M(Handle *h, int f) {
  Freq &q = h->f[f];
  dim3 g((unsigned)((h->ldm + 255) / 256), (unsigned)(h->n + h->E));
  k_merge_M<<<g, 256, 0, h->stream>>>(q.T32, q.y64, q.R64, h->n, h->E, h->ldm, q.M64);
  h->nlaunch += 1;
  return cudaGetLastError();
}

namespace {

// T32 -= A_op B_op^T from the lane's operands (built for K = Kt), on the
// lane's stream; rank is the complex rank the operands carry (for the timing).
cudaError_t launch_c64_tc(Handle *h, int f, int Kt, int rank) {
  Freq &q = h->f[f];
  const long n = h->n;
  cudaError_t e = get_encoder();
  if (e != cudaSuccess) return e;
  Lane &L = lane_of(h, f);
  cudaStream_t st = lane_stream(h, f);
  const int bn = (rank > kAccTuneRank ? h->c64_cols_build : h->c64_cols) == 64 ? 64 : 128;
  const int dcols = (int)(2 * n);
  CUtensorMap ma, mb, md;
  if ((e = make_map(&ma, L.Aop, h->aop_rows, Kt, h->kt_cap, TC_BM)) != cudaSuccess) return e;
  if ((e = make_map(&mb, L.Bop, h->bop_rows, Kt, h->kt_cap, bn)) != cudaSuccess) return e;
  if ((e = make_map(&md, reinterpret_cast<const float *>(q.T32), n, dcols, 2 * h->ldm, TC_BM)) != cudaSuccess)
    return e;
  if (g_c64_sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_c64_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_c64_sms <= 0) g_c64_sms = 1;
  }
  const int ncb = (dcols + bn - 1) / bn, ntiles = ncb * (int)((n + TC_BM - 1) / TC_BM);
  const int grid = persistent_grid(h, ntiles, g_c64_sms);
  if ((e = chain_update_wait(h, f, st)) != cudaSuccess) return e;  // one lane's update at a time
  cudaEvent_t t0 = timing_mark(h, st);
  // long K (build chunks, flushes of deferred updates): one staged tile of T
  // and a deeper operand ring
  const int nkb = Kt / TC_BK;
  const bool longk = nkb >= kLongKStages;
  auto go = [&](auto kern, size_t smem) -> cudaError_t {
    cudaError_t r = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (r != cudaSuccess) return r;
    kern<<<grid, TC_THREADS, smem, st>>>(ma, mb, md, dcols, ncb, ntiles, nkb, h->d_tc_err);
    return cudaGetLastError();
  };
  if (bn == 64)
    e = longk ? go(k_tc_update<64, 1>, C64Tile<64, 1>::SMEM) : go(k_tc_update<64, 2>, C64Tile<64, 2>::SMEM);
  else
    e = longk ? go(k_tc_update<128, 1>, C64Tile<128, 1>::SMEM) : go(k_tc_update<128, 2>, C64Tile<128, 2>::SMEM);
  if (e != cudaSuccess) return e;
  if ((e = chain_update_done(h, f, st)) != cudaSuccess) return e;
  const double cells = (double)n * (double)n;  // complex entries of T updated
  timing_close(h, t0, T_UPDATE, 8.0 * rank * cells,
               2.0 * 8.0 * cells + 4.0 * Kt * ((double)h->aop_rows + (double)h->bop_rows), 0.0, st);
  h->nlaunch += 1;
  return cudaGetLastError();
}

cudaError_t launch_side_update(Handle *h, int f, int k) {
  Freq &q = h->f[f];
  const long n = h->n, rows = n + h->E;
  Lane &L = lane_of(h, f);
  const long side = n + (long)h->E * (n + 1);
  k_c64_side_update<<<(unsigned)((side + 255) / 256), 256, 0, lane_stream(h, f)>>>(q.y64, q.R64, n, h->E, h->ldm,
                                                                                   L.A, rows, L.W, k);
  h->nlaunch += 1;
  return cudaGetLastError();
}

int kt_of(int rank) { return (6 * rank + TC_BK - 1) / TC_BK * TC_BK; }

// Ranks from which updates take the long-K kernel (build chunks, flushes).
constexpr int kLongKRank = 64;
int k2_of(int rank) { return (2 * rank + TC_BK - 1) / TC_BK * TC_BK; }
bool use_longk(const Handle *h, int rank) { return rank >= kLongKRank && 2 * k2_of(rank) <= h->kt_cap; }

// T32 -= A_real B_real^T with the long-K kernel, from the hi / lo operands the
// caller built in the lane's operand buffers (A_hi at Aop, A_lo after it; B
// likewise; leading dimension K2).
cudaError_t launch_c64_tc_longk(Handle *h, int f, int rank) {
  Freq &q = h->f[f];
  const long n = h->n;
  cudaError_t e = get_encoder();
  if (e != cudaSuccess) return e;
  Lane &L = lane_of(h, f);
  cudaStream_t st = lane_stream(h, f);
  const int K2 = k2_of(rank);
  const int dcols = (int)(2 * n);
  float *Ahi = L.Aop, *Alo = L.Aop + (size_t)h->aop_rows * K2;
  float *Bhi = L.Bop, *Blo = L.Bop + (size_t)h->bop_rows * K2;
  CUtensorMap mahi, malo, mbhi, mblo, md;
  if ((e = make_map(&mahi, Ahi, h->aop_rows, K2, K2, TC_BM)) != cudaSuccess ||
      (e = make_map(&malo, Alo, h->aop_rows, K2, K2, TC_BM)) != cudaSuccess ||
      (e = make_map(&mbhi, Bhi, h->bop_rows, K2, K2, LK_BN)) != cudaSuccess ||
      (e = make_map(&mblo, Blo, h->bop_rows, K2, K2, LK_BN)) != cudaSuccess ||
      (e = make_map(&md, reinterpret_cast<const float *>(q.T32), n, dcols, 2 * h->ldm, TC_BM)) != cudaSuccess)
    return e;
  if (g_c64_sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_c64_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_c64_sms <= 0) g_c64_sms = 1;
  }
  const int ncb = (dcols + LK_BN - 1) / LK_BN, ntiles = ncb * (int)((n + TC_BM - 1) / TC_BM);
  const int grid = persistent_grid(h, ntiles, g_c64_sms);
  if ((e = cudaFuncSetAttribute(k_tc_update_longk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)LK_SMEM)) !=
      cudaSuccess)
    return e;
  if ((e = chain_update_wait(h, f, st)) != cudaSuccess) return e;
  cudaEvent_t t0 = timing_mark(h, st);
  k_tc_update_longk<<<grid, LK_THREADS, LK_SMEM, st>>>(mahi, malo, mbhi, mblo, md, dcols, ncb, ntiles, K2 / TC_BK,
                                                        h->d_tc_err);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = chain_update_done(h, f, st)) != cudaSuccess) return e;
  const double cells = (double)n * (double)n;  // complex entries of T updated
  timing_close(h, t0, T_UPDATE, 8.0 * rank * cells,
               2.0 * 8.0 * cells + 2.0 * 4.0 * K2 * ((double)h->aop_rows + (double)h->bop_rows), 0.0, st);
  h->nlaunch += 1;
  return cudaSuccess;
}

}  // namespace

cudaError_t launch_c64_update(Handle *h, int f, int k) {
  const long n = h->n, rows = n + h->E;
  const int Kt = kt_of(k);
  if (Kt > h->kt_cap) return cudaErrorInvalidValue;
  Lane &L = lane_of(h, f);
  cudaStream_t st = lane_stream(h, f);
  cudaError_t e = launch_side_update(h, f, k);  // FP64 side: y and R/Eobj
  if (e != cudaSuccess) return e;
  const size_t sma = sizeof(double2) * (size_t)k * (BO_ROWS + 1), smb = sizeof(double2) * (size_t)k * (BO_COLS + 1);
  if ((e = cudaFuncSetAttribute(k_build_Aop, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sma)) != cudaSuccess)
    return e;
  if (use_longk(h, k)) {  // build chunks: hi / lo operands for the long-K kernel
    const int K2 = k2_of(k);
    if ((e = cudaFuncSetAttribute(k_build_hl_A, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sma)) !=
        cudaSuccess)
      return e;
    k_build_hl_A<<<(unsigned)((n + BO_ROWS - 1) / BO_ROWS), 256, sma, st>>>(L.A, rows, n, k, K2, L.Aop,
                                                                             L.Aop + (size_t)h->aop_rows * K2);
    k_build_hl_B<<<(unsigned)((n + BO_COLS - 1) / BO_COLS), 256, smb, st>>>(L.W, h->ldm, n, k, K2, L.Bop,
                                                                             L.Bop + (size_t)h->bop_rows * K2);
    h->nlaunch += 2;
    return launch_c64_tc_longk(h, f, k);
  }
  k_build_Aop<<<(unsigned)((n + BO_ROWS - 1) / BO_ROWS), 256, sma, st>>>(L.A, rows, n, k, Kt, h->kt_cap, L.Aop);
  k_build_Bop<<<(unsigned)((n + BO_COLS - 1) / BO_COLS), 256, smb, st>>>(L.W, h->ldm, n, k, Kt, h->kt_cap, L.Bop);
  h->nlaunch += 2;
  return launch_c64_tc(h, f, Kt, k);
}

cudaError_t launch_c64_flush(Handle *h, int f) {
  const long n = h->n;
  const int rank = h->defer_rp;
  if (rank <= 0) return cudaSuccess;
  const int Kt = kt_of(rank);
  if (Kt > h->kt_cap) return cudaErrorInvalidValue;
  Freq &q = h->f[f];
  Lane &L = lane_of(h, f);
  cudaStream_t st = lane_stream(h, f);
  if (use_longk(h, rank)) {
    const int K2 = k2_of(rank);
    const dim3 ga((unsigned)((K2 + 127) / 128), (unsigned)n), gb((unsigned)((K2 + 127) / 128), (unsigned)(2 * n));
    k_build_hl_Af<<<ga, 128, 0, st>>>(q.U, h->defer_cap, n, rank, K2, L.Aop, L.Aop + (size_t)h->aop_rows * K2);
    k_build_hl_Bf<<<gb, 128, 0, st>>>(q.Vt, h->defer_cap, n, rank, K2, L.Bop, L.Bop + (size_t)h->bop_rows * K2);
    h->nlaunch += 2;
    return launch_c64_tc_longk(h, f, rank);
  }
  const dim3 ga((unsigned)((Kt + 127) / 128), (unsigned)n), gb((unsigned)((Kt + 127) / 128), (unsigned)(2 * n));
  k_build_Aop_f<<<ga, 128, 0, st>>>(q.U, h->defer_cap, n, rank, Kt, h->kt_cap, L.Aop);
  k_build_Bop_f<<<gb, 128, 0, st>>>(q.Vt, h->defer_cap, n, rank, Kt, h->kt_cap, L.Bop);
  h->nlaunch += 2;
  return launch_c64_tc(h, f, Kt, rank);
}

cudaError_t launch_c64_defer(Handle *h, int f, int k) {
  const long n = h->n, rows = n + h->E;
  Freq &q = h->f[f];
  Lane &L = lane_of(h, f);
  cudaError_t e = launch_side_update(h, f, k);
  if (e != cudaSuccess) return e;
  const size_t sma = sizeof(float2) * 2 * (size_t)k * (DA_ROWS + 1);  // k <= kMaxK: at most 99 KB
  if ((e = cudaFuncSetAttribute(k_defer_append, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sma)) !=
      cudaSuccess)
    return e;
  k_defer_append<<<(unsigned)((n + DA_ROWS - 1) / DA_ROWS), 256, sma, lane_stream(h, f)>>>(
      L.A, rows, L.W, h->ldm, n, k, h->defer_rp, h->defer_cap, q.U, q.Vt);
  h->nlaunch += 1;
  if ((e = cudaGetLastError()) != cudaSuccess || !h->defer_flush) return e;
  const int rp = h->defer_rp;
  h->defer_rp = rp + k;  // the flush covers the accept just appended
  e = launch_c64_flush(h, f);
  h->defer_rp = rp;
  return e;
}

}  // namespace pngf
