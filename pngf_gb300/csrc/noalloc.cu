// Accept step that allocates nothing: pngf_accept_edges_noalloc.
//
// Some callers cannot allocate device memory: a host framework whose caching
// allocator owns the GPU's memory and forbids allocations it does not make,
// an FFI host (JNI, a plugin ABI) that has no way to free device memory it did
// not allocate itself, or a hot loop where the device-wide synchronisation of
// cudaMalloc/cudaFree is not acceptable. The handle API allocates its scratch
// in pngf_create; this entry point instead works on buffers the caller owns
// and keeps its scratch (the LU factors, pivots, z, the gathered columns A and
// the right-hand factor W of the rank-k update) in one file-scope device array
// of fixed size, kScratchBytes (8 MiB), which every GPU that loads this
// library holds until the process exits.
//
// Set-up: the first call on each device, with that device current, looks up
// the array's device address with cudaGetSymbolAddress and caches it; make
// that first call before any stream capture. The cached address belongs to
// the device's primary context: after cudaDeviceReset the module is loaded
// again and the array may move, so this entry point must not be used across a
// device reset. All calls share the one array and it keeps the last call's
// contents: calls that overlap on the GPU (on different streams, or from
// several host threads) race on it, so serialise them on one stream.
//
// The caller's edge list is untrusted input: the factor kernel checks every
// index against [0, n) and every sign against +-1 before any of them
// addresses M, and on a bad entry sets the status to PNGF_ERR_ARG; on a
// singular K it sets PNGF_ERR_SINGULAR. In both cases the later kernels return
// without writing, so M is left exactly as it was. The status word (the
// caller's, or one inside the scratch array when status is NULL) is cleared
// at the start of every call.
#include <cuda_runtime.h>

#include <mutex>

#include "pngf_internal.h"

namespace {

constexpr size_t kScratchBytes = size_t(8) << 20;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_scratch[kScratchBytes];

std::mutex g_mu;
void *g_scratch_ptr[kMaxDevices];

size_t align256(size_t b) { return (b + 255) / 256 * 256; }

}  // namespace

extern "C" int pngf_accept_edges_noalloc(double *M, long ldm, long n, int num_eobj, const double *Einc,
                                         const int *s, const signed char *d, int k, int *status, void *stream) {
  if (!M || !Einc || !s || !d || n <= 0 || ldm < n + 1 || num_eobj < 1 || num_eobj > PNGF_MAX_EOBJ)
    return PNGF_ERR_ARG;
  if (k < 0 || k > pngf::kMaxEvalK) return PNGF_ERR_ARG;
  if (k == 0) return PNGF_OK;
  // Scratch layout: status | LU (k x k) | piv (k) | z (k) | A ((n+E) x k) | W (k x ldm).
  const size_t o_status = 0;
  const size_t o_lu = align256(sizeof(int));
  const size_t o_piv = o_lu + align256(sizeof(double2) * (size_t)k * k);
  const size_t o_z = o_piv + align256(sizeof(int) * (size_t)k);
  const size_t o_a = o_z + align256(sizeof(double2) * (size_t)k);
  const size_t o_w = o_a + align256(sizeof(double2) * (size_t)(n + num_eobj) * k);
  const size_t need = o_w + align256(sizeof(double2) * (size_t)k * ldm);
  if (need > kScratchBytes) return PNGF_ERR_SCRATCH;

  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return PNGF_ERR_NO_DEVICE;
  unsigned char *base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_ptr[dev]) {
      void *p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
      if (e != cudaSuccess || !p) {
        cudaGetLastError();
        return PNGF_ERR_CUDA;
      }
      g_scratch_ptr[dev] = p;
    }
    base = static_cast<unsigned char *>(g_scratch_ptr[dev]);
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int *d_status = status ? status : reinterpret_cast<int *>(base + o_status);
  if (cudaMemsetAsync(d_status, 0, sizeof(int), st) != cudaSuccess) return PNGF_ERR_CUDA;
  const cudaError_t e = pngf::launch_accept_raw(
      reinterpret_cast<double2 *>(M), ldm, n, num_eobj, reinterpret_cast<const double2 *>(Einc), s, d, k,
      reinterpret_cast<double2 *>(base + o_lu), reinterpret_cast<int *>(base + o_piv),
      reinterpret_cast<double2 *>(base + o_z), reinterpret_cast<double2 *>(base + o_a),
      reinterpret_cast<double2 *>(base + o_w), d_status, st);
  return e == cudaSuccess ? PNGF_OK : PNGF_ERR_CUDA;
}
