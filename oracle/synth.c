/* Synthetic G and NF2FF rows, restated in C (test infrastructure only).
 *
 * The inputs of every oracle run: a stand-in for acmefdfd's per-frequency
 * G file, which cannot be produced here (its MUMPS/APF Schur precompute
 * needs MUMPS, MPI and METIS). The tests, the golden-log generator and the
 * CPU legs of bench.py build G with this file so that no oracle run loads the
 * library under test; a test checks that the library's own generator gives
 * the same matrices.
 *
 * Edge (DOF) numbering follows pngf-opt/pngfopt.hpp:86-94 and 640-661: all
 * Ex edges first, x fastest, on a (tx*cx) x (ty*cy+1) grid, centred at
 * ((i+1/2) dx, j dy); then all Ey edges on a (tx*cx+1) x (ty*cy) grid,
 * centred at (i dx, (j+1/2) dy).
 *
 * G (n x n, column-major): between edge centres, the free-space dyadic
 * Helmholtz Green's function at k = 2 pi f sqrt(eps_r) / c0 in
 * electric-field form, i w mu0 dV (I + grad grad / k^2) e^{ikR} / (4 pi R),
 * projected on the two edge directions; diagonal (0.3 + 0.05i) times the
 * largest off-diagonal magnitude of its column; every entry then times
 * (1 + 1e-3 g_ij), g a unit-variance complex Gaussian of the unordered pair
 * {i, j} (splitmix64 counter hash, Box-Muller). Complex-symmetric.
 *
 * NF2FF rows (2 x n, row-major: the rows N and N+1 of an acmefdfd G file,
 * acmefdfd/main.cpp:466-492, read by pngfopt.hpp:173-180): the broadside
 * (theta = phi = 0) far-field projection of the edge currents, theta
 * polarisation (x-directed edges) in row 1 and phi polarisation (y-directed
 * edges) in row 2; at broadside the phase of a planar source is constant, so
 * an edge's entry is the amplitude kappa eta0 dV for its own polarisation and
 * 0 for the other, times (1 + 1e-3 q), q a unit complex Gaussian of the
 * pair {e, n + row}. kappa = 32 makes the directivity term of the objective
 * O(1) on this G (whose port resistance is not a physical one).
 *
 * Built without -ffast-math so that the arithmetic follows IEEE order.
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>

typedef double complex zc;

static const double kC0 = 2.997924579998211e8;  /* pngf-opt/main.cpp:101 */
static const double kMu0 = 1.25663706127e-6;
static const double kEta0 = 3.767303134118051e02; /* pngf-opt/main.cpp:102 */
static const double kKappa = 32.0;
static const double kPi = 3.14159265358979323846;

typedef struct {
  long n, nx;
  int ex_xsz, ey_xsz;
  double dx, dy;
} geo_t;

static geo_t make_geo(int tx, int ty, int cx, int cy, double dx, double dy) {
  geo_t g;
  g.ex_xsz = tx * cx;
  g.ey_xsz = tx * cx + 1;
  g.nx = (long)g.ex_xsz * (ty * cy + 1);
  g.n = g.nx + (long)g.ey_xsz * (ty * cy);
  g.dx = dx;
  g.dy = dy;
  return g;
}

static void centre(const geo_t *g, long e, double *x, double *y, int *dir) {
  if (e < g->nx) {
    const long iy = e / g->ex_xsz, ix = e - iy * g->ex_xsz;
    *x = (ix + 0.5) * g->dx;
    *y = iy * g->dy;
    *dir = 0;
  } else {
    const long q = e - g->nx, iy = q / g->ey_xsz, ix = q - iy * g->ey_xsz;
    *x = ix * g->dx;
    *y = (iy + 0.5) * g->dy;
    *dir = 1;
  }
}

static uint64_t mix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

/* Unit-variance complex Gaussian of the unordered pair {i, j}. */
static zc pair_gauss(uint64_t seed, uint64_t i, uint64_t j) {
  if (i > j) {
    const uint64_t t = i;
    i = j;
    j = t;
  }
  const uint64_t h = mix64(seed * 0x2545F4914F6CDD1Dull ^ mix64(i * 0x100000001B3ull + j));
  const uint64_t h2 = mix64(h);
  const double u1 = ((h >> 11) + 1) * (1.0 / 9007199254740992.0); /* (0, 1] */
  const double u2 = (h2 >> 11) * (1.0 / 9007199254740992.0);      /* [0, 1) */
  const double r = sqrt(-2.0 * log(u1));
  const double t = 2.0 * kPi * u2;
  const double s = 0.70710678118654752440;
  return r * cos(t) * s + I * (r * sin(t) * s);
}

long synth_num_edges(int tx, int ty, int cx, int cy) { return make_geo(tx, ty, cx, cy, 1.0, 1.0).n; }

/* G into out (column-major, leading dimension ld >= n). Returns n, or -1. */
long synth_G(int tx, int ty, int cx, int cy, double dx, double dy, double dz, double freq_hz, double eps_r,
             unsigned long long seed, double *out, long ld) {
  const geo_t g = make_geo(tx, ty, cx, cy, dx, dy);
  const long n = g.n;
  if (tx <= 0 || ty <= 0 || cx <= 0 || cy <= 0 || !out || ld < n) return -1;
  const double k = 2.0 * kPi * freq_hz * sqrt(eps_r) / kC0;
  const double w_mu_dv = 2.0 * kPi * freq_hz * kMu0 * dx * dy * dz;
  zc *G = (zc *)out;
  double *colmax = (double *)calloc((size_t)n, sizeof(double));
  if (!colmax) return -1;
#pragma omp parallel for schedule(dynamic, 16)
  for (long j = 0; j < n; ++j) {
    double xj, yj, m = 0.0;
    int dj;
    centre(&g, j, &xj, &yj, &dj);
    zc *col = G + (size_t)j * ld;
    for (long i = 0; i < n; ++i) {
      if (i == j) {
        col[i] = 0.0;
        continue;
      }
      double xi, yi;
      int di;
      centre(&g, i, &xi, &yi, &di);
      const double rx = xi - xj, ry = yi - yj;
      const double R = sqrt(rx * rx + ry * ry);
      const double kr = k * R;
      /* (1 + i/kr - 1/kr^2) delta_ij + (-1 - 3i/kr + 3/kr^2) (u_i . Rhat)(u_j . Rhat) */
      const double a_re = 1.0 - 1.0 / (kr * kr), a_im = 1.0 / kr;
      const double b_re = -1.0 + 3.0 / (kr * kr), b_im = -3.0 / kr;
      const double ui = di == 0 ? rx / R : ry / R;
      const double uj = dj == 0 ? rx / R : ry / R;
      const double dd = di == dj ? 1.0 : 0.0;
      const double uu = ui * uj;
      const double inv = 1.0 / (4.0 * kPi * R);
      const zc phase = cos(kr) * inv + I * (sin(kr) * inv);
      const zc t = (a_re * dd + b_re * uu) + I * (a_im * dd + b_im * uu);
      const zc v = (I * w_mu_dv) * phase * t;
      col[i] = v;
      const double av = cabs(v);
      if (av > m) m = av;
    }
    colmax[j] = m;
  }
#pragma omp parallel for schedule(dynamic, 16)
  for (long j = 0; j < n; ++j) {
    zc *col = G + (size_t)j * ld;
    col[j] = (0.3 + 0.05 * I) * colmax[j];
    for (long i = 0; i < n; ++i) col[i] *= 1.0 + 1e-3 * pair_gauss(seed, (uint64_t)i, (uint64_t)j);
  }
  free(colmax);
  return n;
}

/* The two NF2FF rows into rows (2 x n complex, row-major). Returns n, or -1. */
long synth_gobj(int tx, int ty, int cx, int cy, double dx, double dy, double dz, unsigned long long seed,
                double *rows) {
  const geo_t g = make_geo(tx, ty, cx, cy, dx, dy);
  const long n = g.n;
  if (tx <= 0 || ty <= 0 || cx <= 0 || cy <= 0 || !rows) return -1;
  const double amp = kKappa * kEta0 * dx * dy * dz;
  zc *r = (zc *)rows;
  for (int row = 0; row < 2; ++row)
    for (long e = 0; e < n; ++e) {
      const int dir = e < g.nx ? 0 : 1;
      r[(size_t)row * n + e] =
          dir == row ? amp * (1.0 + 1e-3 * pair_gauss(seed, (uint64_t)e, (uint64_t)(n + row))) : 0.0;
    }
  return n;
}
