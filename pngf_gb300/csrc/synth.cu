// Synthetic G (and its NF2FF rows) generated on the device.
//
// The same recipe as the host generator in gfile.cpp (pngf_synth_G): the
// free-space dyadic Helmholtz Green's function between Yee edge centres in
// electric-field form (i w mu0 dV scale), diagonal (0.3 + 0.05i) times the
// largest off-diagonal magnitude of its column, and a seeded symmetric
// complex Gaussian relative perturbation of 1e-3 per unordered edge pair.
// The device's sqrt, exp, sin, cos and log round differently from the host
// C library's in the last bits, so entries agree with the host generator to
// about 1e-15 relative, not bit for bit.
//
// Used where G would not fit in host memory or take minutes to generate on
// the host: large maps and many-instance runs whose handles keep only their
// state on the device and regenerate G when a build or drift check needs it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>

#include "pngf_internal.h"

namespace pngf {
namespace {

struct SynthGeo {
  long n, nx;
  int ex_xsz, ey_xsz;
  double dx, dy;
  double k;           // wavenumber
  double sre, sim;    // i w mu0 dV
  unsigned long long seed;
};

__device__ __forceinline__ void edge_centre(const SynthGeo &g, long e, double *x, double *y, int *dir) {
  if (e < g.nx) {
    const long iy = e / g.ex_xsz, ix = e - iy * g.ex_xsz;
    *x = (ix + 0.5) * g.dx;
    *y = iy * g.dy;
    *dir = 0;
  } else {
    const long q = e - g.nx, iy = q / g.ey_xsz, ix = q - iy * g.ey_xsz;
    *x = ix * g.dx;
    *y = (iy + 0.5) * g.dy;
    *dir = 1;
  }
}

__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// Unit-variance complex Gaussian of the unordered pair {i, j} (Box-Muller).
__device__ double2 pair_gaussian(uint64_t seed, uint64_t i, uint64_t j) {
  if (i > j) {
    const uint64_t t = i;
    i = j;
    j = t;
  }
  const uint64_t h = splitmix64(seed * 0x2545F4914F6CDD1Dull ^ splitmix64(i * 0x100000001B3ull + j));
  const uint64_t h2 = splitmix64(h);
  const double u1 = ((h >> 11) + 1) * (1.0 / 9007199254740992.0);
  const double u2 = (h2 >> 11) * (1.0 / 9007199254740992.0);
  const double r = sqrt(-2.0 * log(u1));
  const double t = 2.0 * M_PI * u2;
  double s, c;
  sincos(t, &s, &c);
  return make_double2(r * c * M_SQRT1_2, r * s * M_SQRT1_2);
}

__device__ __forceinline__ double2 zmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// One off-diagonal entry (0 on the diagonal).
__device__ double2 offdiag_entry(const SynthGeo &g, long i, long j) {
  if (i == j) return make_double2(0.0, 0.0);
  double xi, yi, xj, yj;
  int di, dj;
  edge_centre(g, i, &xi, &yi, &di);
  edge_centre(g, j, &xj, &yj, &dj);
  const double rx = xi - xj, ry = yi - yj;
  const double R = sqrt(rx * rx + ry * ry);
  const double kr = g.k * R;
  const double ikr = 1.0 / kr, ikr2 = 1.0 / (kr * kr);
  const double2 a = make_double2(1.0 - ikr2, ikr);
  const double2 b = make_double2(-1.0 + 3.0 * ikr2, -3.0 * ikr);
  const double ui = di == 0 ? rx / R : ry / R;  // edge i direction . Rhat
  const double uj = dj == 0 ? rx / R : ry / R;  // edge j direction . Rhat
  const double dd = di == dj ? 1.0 : 0.0;
  const double uu = ui * uj;
  double s, c;
  sincos(kr, &s, &c);
  const double inv = 1.0 / (4.0 * M_PI * R);
  const double2 phase = make_double2(c * inv, s * inv);
  const double2 t = make_double2(a.x * dd + b.x * uu, a.y * dd + b.y * uu);
  return zmul(zmul(make_double2(g.sre, g.sim), phase), t);
}

// Off-diagonal entries, rows along x and columns along y (in steps of
// gridDim.y), and each column's largest magnitude into colmax (non-negative
// doubles' bits order like unsigned integers: atomic max).
__global__ void k_synth_offdiag(double2 *__restrict__ G, long ldg, SynthGeo g,
                                unsigned long long *__restrict__ colmax) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  for (long j = blockIdx.y; j < g.n; j += gridDim.y) {
    double m = 0.0;
    if (i < g.n) {
      const double2 v = offdiag_entry(g, i, j);
      G[(size_t)j * ldg + i] = v;
      m = hypot(v.x, v.y);
    }
    for (int o = 16; o; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(colmax + j, (unsigned long long)__double_as_longlong(m));
  }
}

// Diagonal (0.3 + 0.05i) colmax, then every entry times 1 + 1e-3 g_ij.
__global__ void k_synth_finish(double2 *__restrict__ G, long ldg, SynthGeo g,
                               const unsigned long long *__restrict__ colmax) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n) return;
  for (long j = blockIdx.y; j < g.n; j += gridDim.y) {
    double2 v;
    if (i == j) {
      const double m = __longlong_as_double((long long)colmax[j]);
      v = make_double2(0.3 * m, 0.05 * m);
    } else {
      v = G[(size_t)j * ldg + i];
    }
    const double2 p = pair_gaussian(g.seed, (uint64_t)i, (uint64_t)j);
    G[(size_t)j * ldg + i] = zmul(v, make_double2(1.0 + 1e-3 * p.x, 1e-3 * p.y));
  }
}

// The NF2FF rows of the synthetic G (the recipe of pngf_synth_gobj): row 1
// (theta polarisation at broadside) amp on x-directed edges, row 2 (phi) amp
// on y-directed edges, each entry times 1 + 1e-3 q, q the complex Gaussian of
// the pair {e, n + row}; any further rows zero.
__global__ void k_synth_gobj(double2 *__restrict__ rows, int nrows, SynthGeo g, double amp) {
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const int row = blockIdx.y;
  if (e >= g.n || row >= nrows) return;
  const int dir = e < g.nx ? 0 : 1;
  double2 v = make_double2(0.0, 0.0);
  if (row < 2 && dir == row) {
    const double2 q = pair_gaussian(g.seed, (uint64_t)e, (uint64_t)(g.n + row));
    v = make_double2(amp * (1.0 + 1e-3 * q.x), amp * (1e-3 * q.y));
  }
  rows[(size_t)row * g.n + e] = v;
}

}  // namespace

cudaError_t launch_synth_gobj(Handle *h, int f, double2 *rows) {
  if (h->E <= 1) return cudaSuccess;
  SynthGeo g{};
  g.n = h->n;
  g.nx = h->nx;
  g.seed = h->f[f].synth_seed;
  const dim3 grid((unsigned)((h->n + 255) / 256), (unsigned)(h->E - 1));
  k_synth_gobj<<<grid, 256, 0, h->stream>>>(rows, h->E - 1, g, synth_gobj_amplitude(h->cfg.dx, h->cfg.dy, h->cfg.dz));
  h->nlaunch += 1;
  return cudaGetLastError();
}

cudaError_t launch_synth_G(Handle *h, int f, double2 *G, long ldg, unsigned long long *colmax) {
  const Freq &q = h->f[f];
  SynthGeo g;
  g.n = h->n;
  g.nx = h->nx;
  g.ex_xsz = h->ex_xsz;
  g.ey_xsz = h->ey_xsz;
  g.dx = h->cfg.dx;
  g.dy = h->cfg.dy;
  const double c0 = 2.997924579998211e8, mu0 = 1.25663706127e-6;
  const double fr = h->cfg.freq_hz[f];
  g.k = 2.0 * M_PI * fr * std::sqrt(q.synth_eps) / c0;
  g.sre = 0.0;
  g.sim = 2.0 * M_PI * fr * mu0 * h->cfg.dx * h->cfg.dy * h->cfg.dz;
  g.seed = q.synth_seed;
  cudaError_t e = cudaMemsetAsync(colmax, 0, sizeof(unsigned long long) * h->n, h->stream);
  if (e != cudaSuccess) return e;
  const dim3 grid((unsigned)((h->n + 255) / 256), (unsigned)std::min<long>(h->n, 65535));
  k_synth_offdiag<<<grid, 256, 0, h->stream>>>(G, ldg, g, colmax);
  k_synth_finish<<<grid, 256, 0, h->stream>>>(G, ldg, g, colmax);
  h->nlaunch += 2;
  return cudaGetLastError();
}

}  // namespace pngf
