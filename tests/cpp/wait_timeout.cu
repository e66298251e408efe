// The failure path of the tensor-core kernels' bounded waits, on a wait that
// nothing completes: an mbarrier that expects one arrival which never comes,
// waited on with the library's own bounded wait (suspending tries, a limit on
// the global timer) given a short limit. The kernel must give up, record an
// error code, and leave the context usable (a second kernel then runs and its
// result is read back).
#include <cstdio>
#include <cstdlib>

#include "../../pngf_gb300/csrc/tc_common.cuh"

using namespace pngf::tc;

__global__ void k_wait_nothing(unsigned long long limit_ns, int *err) {
  __shared__ uint64_t bar;
  const uint32_t b = smem_u32(&bar);
  if (threadIdx.x == 0) {
    mbar_init(b, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const unsigned long long t0 = global_ns();
  const bool ok = mbar_wait_for(b, 0, limit_ns);
  const unsigned long long waited = global_ns() - t0;
  if (!ok && threadIdx.x == 0) {
    atomicExch(err, 77);
    err[2] = (int)(waited / 1000);  // microseconds spent waiting
  }
}

__global__ void k_after(int *out) { *out = 1234; }

int main(int argc, char **argv) {
  const unsigned long long limit_us = argc > 1 ? (unsigned long long)atoll(argv[1]) : 20000ull;
  int *d = nullptr;
  if (cudaMalloc(&d, 3 * sizeof(int)) != cudaSuccess) return 2;
  cudaMemset(d, 0, 3 * sizeof(int));
  k_wait_nothing<<<1, 32>>>(limit_us * 1000ull, d);
  cudaError_t e1 = cudaDeviceSynchronize();
  k_after<<<1, 1>>>(d + 1);
  cudaError_t e2 = cudaDeviceSynchronize();
  int h[3] = {0, 0, 0};
  cudaError_t e3 = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
  printf("wait status %d, after %d, waited_us %d, cuda %s %s %s\n", h[0], h[1], h[2], cudaGetErrorString(e1),
         cudaGetErrorString(e2), cudaGetErrorString(e3));
  cudaFree(d);
  return (e1 == cudaSuccess && e2 == cudaSuccess && e3 == cudaSuccess && h[0] == 77 && h[1] == 1234) ? 0 : 1;
}
