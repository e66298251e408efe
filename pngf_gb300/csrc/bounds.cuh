// Bounds-checked build (compile with -DPNGF_BOUNDS_CHECK; python -m
// pngf_gb300.build --bounds-check writes libpngf_gb300_bc.so).
//
// The kernels whose addresses depend on data -- the gathers of M through edge
// lists built on the device (candidate kernels, the accept's factor, W solves
// and column gathers, the row gather of the tensor-core W product) and the
// reads of Einc by edge -- check every data-dependent index against the
// extent it addresses. A violation is recorded (count, then kind, row and
// column of the first one) in a device word of the translation unit, the
// access is skipped and reads as zero; nothing traps. The host reads the
// record with pngf_bounds_check_report. This stands in for compute-sanitizer
// on pools where it is closed: the parity tests run on this build and must
// record no violation. In the default build the checks compile to nothing.
#pragma once

#include <cuda_runtime.h>

namespace pngf {

enum BoundsKind { kBoundsT = 1, kBoundsY = 2, kBoundsR = 3, kBoundsEinc = 4, kBoundsRowIdx = 5 };

#ifdef PNGF_BOUNDS_CHECK
// One record per translation unit (no relocatable device code): count, kind,
// row, column of the first violation.
static __device__ unsigned long long g_bounds_rec[4];

__device__ __noinline__ inline void bounds_fail(int kind, long long i, long long j) {
  if (atomicAdd(&g_bounds_rec[0], 1ull) == 0ull) {
    g_bounds_rec[1] = (unsigned long long)kind;
    g_bounds_rec[2] = (unsigned long long)i;
    g_bounds_rec[3] = (unsigned long long)j;
  }
}
#define PNGF_BOUNDS_OK(cond, kind, i, j) ((cond) ? true : (::pngf::bounds_fail((kind), (i), (j)), false))

// Reads this translation unit's record into out[4] and clears it if reset.
static inline cudaError_t bounds_read_tu(long long out[4], bool reset) {
  unsigned long long v[4];
  cudaError_t e = cudaMemcpyFromSymbol(v, g_bounds_rec, sizeof(v));
  if (e != cudaSuccess) return e;
  for (int q = 0; q < 4; ++q) out[q] = (long long)v[q];
  if (reset) {
    const unsigned long long z[4] = {0, 0, 0, 0};
    e = cudaMemcpyToSymbol(g_bounds_rec, z, sizeof(z));
  }
  return e;
}
#else
#define PNGF_BOUNDS_OK(cond, kind, i, j) true
#endif

// Per translation unit readers (bounds-checked build only; each returns the
// record of the kernels in its file).
cudaError_t bounds_read_fp64(long long out[4], bool reset);
cudaError_t bounds_read_f64tc(long long out[4], bool reset);

}  // namespace pngf
