// G matrices: the acmefdfd file layout and the synthetic stand-in generator.
//
// File layout (written by acmefdfd/main.cpp:533-538, read back by
// pngf-opt/pngfopt.hpp:163-180): one file per frequency holding an
// (N+E-1) x (N+E-1) complex128 matrix in column-major order. The top-left
// N x N block is G over the design edges; rows N .. N+E-2 are the objective
// rows 1 .. E-1 of Gobj (the near-field to far-field rows). Row 0 of Gobj is
// not in the file: it is built from the port (pngfopt.hpp:559-618).
//
// Edge (DOF) ordering, from pngf-opt/pngfopt.hpp:86-94 and 640-661: all Ex
// edges first, x fastest, on a (tx*cx) x (ty*cy+1) grid; then all Ey edges,
// x fastest, on a (tx*cx+1) x (ty*cy) grid.
//
// Synthetic G (the stand-in used when acmefdfd's MUMPS precompute cannot
// run): free-space dyadic Helmholtz Green's function between Yee edge centres,
// projected on the two edge directions and scaled by the cell volume
// dx*dy*dz, in SI units and in electric-field form E = i w mu0 Gd J dV, so
// that G has the units of acmefdfd's G (field per design current density;
// acmefdfd/main.cpp:431-447 scales its right-hand side by 1/(i eps0 w)). The
// diagonal is (0.3+0.05i) times the largest
// off-diagonal magnitude in its row; every entry then gets a seeded symmetric
// complex Gaussian relative perturbation of 1e-3. The result is
// complex-symmetric.
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "pngf_internal.h"

namespace {

struct EdgeGeom {
  double x, y;   // centre, metres
  int dir;       // 0 = x-directed, 1 = y-directed
};

std::vector<EdgeGeom> edge_geometry(int tiles_x, int tiles_y, int cells_x, int cells_y,
                                    double dx, double dy) {
  const int ex_xsz = tiles_x * cells_x, ex_ysz = tiles_y * cells_y + 1;
  const int ey_xsz = tiles_x * cells_x + 1, ey_ysz = tiles_y * cells_y;
  std::vector<EdgeGeom> e;
  e.reserve((size_t)ex_xsz * ex_ysz + (size_t)ey_xsz * ey_ysz);
  for (int iy = 0; iy < ex_ysz; ++iy)
    for (int ix = 0; ix < ex_xsz; ++ix) e.push_back({(ix + 0.5) * dx, iy * dy, 0});
  for (int iy = 0; iy < ey_ysz; ++iy)
    for (int ix = 0; ix < ey_xsz; ++ix) e.push_back({ix * dx, (iy + 0.5) * dy, 1});
  return e;
}

inline uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// Unit-variance complex Gaussian for the unordered pair {i, j}.
inline std::complex<double> pair_gaussian(uint64_t seed, uint64_t i, uint64_t j) {
  if (i > j) std::swap(i, j);
  uint64_t h = splitmix64(seed * 0x2545F4914F6CDD1Dull ^ splitmix64(i * 0x100000001B3ull + j));
  uint64_t h2 = splitmix64(h);
  double u1 = ((h >> 11) + 1) * (1.0 / 9007199254740992.0);  // (0, 1]
  double u2 = (h2 >> 11) * (1.0 / 9007199254740992.0);       // [0, 1)
  double r = std::sqrt(-2.0 * std::log(u1));
  double t = 2.0 * M_PI * u2;
  return {r * std::cos(t) * M_SQRT1_2, r * std::sin(t) * M_SQRT1_2};
}

}  // namespace

extern "C" long pngf_num_edges(int tiles_x, int tiles_y, int cells_x, int cells_y) {
  return (long)(tiles_x * cells_x) * (tiles_y * cells_y + 1) +
         (long)(tiles_x * cells_x + 1) * (tiles_y * cells_y);
}

extern "C" int pngf_synth_G(int tiles_x, int tiles_y, int cells_x, int cells_y, double dx,
                            double dy, double dz, double freq_hz, double eps_r,
                            unsigned long long seed, double *out, long ld) {
  if (tiles_x <= 0 || tiles_y <= 0 || cells_x <= 0 || cells_y <= 0 || !out) return PNGF_ERR_ARG;
  const std::vector<EdgeGeom> e = edge_geometry(tiles_x, tiles_y, cells_x, cells_y, dx, dy);
  const long n = (long)e.size();
  if (ld < n) return PNGF_ERR_ARG;
  const double c0 = 2.997924579998211e8;
  const double k = 2.0 * M_PI * freq_hz * std::sqrt(eps_r) / c0;
  const double mu0 = 1.25663706127e-6;
  const std::complex<double> scale(0.0, 2.0 * M_PI * freq_hz * mu0 * dx * dy * dz);  // i w mu0 dV
  std::complex<double> *g = reinterpret_cast<std::complex<double> *>(out);
  std::vector<double> rowmax(n, 0.0);
#pragma omp parallel for schedule(dynamic, 16)
  for (long j = 0; j < n; ++j) {
    std::complex<double> *col = g + (size_t)j * ld;
    for (long i = 0; i < n; ++i) {
      if (i == j) {
        col[i] = 0.0;
        continue;
      }
      const double rx = e[i].x - e[j].x, ry = e[i].y - e[j].y;
      const double R = std::sqrt(rx * rx + ry * ry);
      const double kr = k * R;
      const std::complex<double> ikr(0.0, 1.0 / kr);
      const std::complex<double> a = 1.0 + ikr - 1.0 / (kr * kr);
      const std::complex<double> b = -1.0 - 3.0 * ikr + 3.0 / (kr * kr);
      const double ui = e[i].dir == 0 ? rx / R : ry / R;  // edge i direction . Rhat
      const double uj = e[j].dir == 0 ? rx / R : ry / R;  // edge j direction . Rhat
      const double dd = e[i].dir == e[j].dir ? 1.0 : 0.0;
      const std::complex<double> phase = std::exp(std::complex<double>(0.0, kr)) / (4.0 * M_PI * R);
      col[i] = scale * phase * (a * dd + b * (ui * uj));  // ui*uj first: bit-symmetric in (i, j)
    }
  }
  // Row maxima (G is symmetric before the diagonal is set, so column maxima
  // are row maxima).
#pragma omp parallel for
  for (long j = 0; j < n; ++j) {
    double m = 0.0;
    const std::complex<double> *col = g + (size_t)j * ld;
    for (long i = 0; i < n; ++i) m = std::max(m, std::abs(col[i]));
    rowmax[j] = m;
  }
#pragma omp parallel for schedule(dynamic, 16)
  for (long j = 0; j < n; ++j) {
    std::complex<double> *col = g + (size_t)j * ld;
    col[j] = std::complex<double>(0.3, 0.05) * rowmax[j];
    for (long i = 0; i < n; ++i) col[i] *= 1.0 + 1e-3 * pair_gaussian(seed, i, j);
  }
  return PNGF_OK;
}

// The two NF2FF rows of the synthetic G (rows N and N+1 of an acmefdfd G file,
// acmefdfd/main.cpp:466-492): the broadside (theta = phi = 0) far-field
// projection of the edge currents. Row 1 (theta polarisation) weights the
// x-directed edges, row 2 (phi) the y-directed ones; a planar source's phase
// is constant at broadside, so each entry is the amplitude kappa eta0 dx dy dz
// (kappa = 32: a directivity term of order one on this G) for its own
// polarisation and zero for the other, times 1 + 1e-3 q with q the complex
// Gaussian of the pair {e, n + row} (the G perturbation's hash, on indices
// that no entry of G uses).
extern "C" int pngf_synth_gobj(int tiles_x, int tiles_y, int cells_x, int cells_y, double dx, double dy,
                               double dz, unsigned long long seed, double *rows) {
  if (tiles_x <= 0 || tiles_y <= 0 || cells_x <= 0 || cells_y <= 0 || !rows) return PNGF_ERR_ARG;
  const long n = pngf_num_edges(tiles_x, tiles_y, cells_x, cells_y);
  const long nx = (long)(tiles_x * cells_x) * (tiles_y * cells_y + 1);
  const double amp = pngf::synth_gobj_amplitude(dx, dy, dz);
  std::complex<double> *r = reinterpret_cast<std::complex<double> *>(rows);
  for (int row = 0; row < 2; ++row)
    for (long e = 0; e < n; ++e) {
      const int dir = e < nx ? 0 : 1;
      r[(size_t)row * n + e] =
          dir == row ? amp * (1.0 + 1e-3 * pair_gaussian(seed, (uint64_t)e, (uint64_t)(n + row))) : 0.0;
    }
  return PNGF_OK;
}

// Writes one G file in the acmefdfd layout. gobj_rows holds num_eobj-1 rows of
// n entries each (row-major, may be NULL for zero rows).
extern "C" int pngf_write_G_file(const char *path, long n, int num_eobj, const double *G,
                                 long ldg, const double *gobj_rows) {
  if (!path || !G || n <= 0 || num_eobj < 1 || ldg < n) return PNGF_ERR_ARG;
  const long m = n + num_eobj - 1;
  FILE *f = std::fopen(path, "wb");
  if (!f) return PNGF_ERR_IO;
  std::vector<std::complex<double>> col(m);
  const std::complex<double> *g = reinterpret_cast<const std::complex<double> *>(G);
  const std::complex<double> *go = reinterpret_cast<const std::complex<double> *>(gobj_rows);
  int rc = PNGF_OK;
  for (long j = 0; j < m && rc == PNGF_OK; ++j) {
    for (long i = 0; i < m; ++i) {
      std::complex<double> v = 0.0;
      if (j < n && i < n) v = g[(size_t)j * ldg + i];
      else if (j < n && go) v = go[(size_t)(i - n) * n + j];
      col[i] = v;
    }
    if (std::fwrite(col.data(), sizeof(col[0]), m, f) != (size_t)m) rc = PNGF_ERR_IO;
  }
  if (std::fclose(f) != 0) rc = PNGF_ERR_IO;
  return rc;
}

// Reads one G file in the acmefdfd layout: G (n x n, column-major, leading
// dimension ldg) and the num_eobj-1 objective rows (row-major, n each).
// A short or missing file is an error (the reference prints and continues,
// pngfopt.hpp:122-127; here the caller gets PNGF_ERR_IO).
extern "C" int pngf_read_G_file(const char *path, long n, int num_eobj, double *G, long ldg,
                                double *gobj_rows) {
  if (!path || !G || n <= 0 || num_eobj < 1 || ldg < n) return PNGF_ERR_ARG;
  const long m = n + num_eobj - 1;
  FILE *f = std::fopen(path, "rb");
  if (!f) return PNGF_ERR_IO;
  std::vector<std::complex<double>> col(m);
  std::complex<double> *g = reinterpret_cast<std::complex<double> *>(G);
  std::complex<double> *go = reinterpret_cast<std::complex<double> *>(gobj_rows);
  int rc = PNGF_OK;
  for (long j = 0; j < n; ++j) {
    if (std::fread(col.data(), sizeof(col[0]), m, f) != (size_t)m) {
      rc = PNGF_ERR_IO;
      break;
    }
    std::memcpy(g + (size_t)j * ldg, col.data(), sizeof(col[0]) * n);
    if (go)
      for (long r = 0; r < num_eobj - 1; ++r) go[(size_t)r * n + j] = col[n + r];
  }
  std::fclose(f);
  return rc;
}
