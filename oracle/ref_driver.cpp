// Oracle driver around the reference optimizer (test infrastructure only).
//
// Compiles the reference's own pngf-opt/{acmetime,linalg,pngfopt,magichat}.hpp
// unmodified (included from the reference tree by the Makefile in this
// directory) and restates the DBS loop of pngf-opt/main.cpp:131-490 with
// the constants that main.cpp hard-codes turned into command-line options:
// tile-map size, frequencies and G files, RNG seed, initial design, candidate
// mode and an evaluation cap. Every evaluated flip is written with 17
// significant digits so that the GPU path can be compared bit-for-bit where
// it should be and to 1e-10 relative where rounding differs.
//
// Candidate modes:
//   sym    - the reference's 4-fold mirror-symmetric quarter hat
//            (main.cpp:181, 343-392), unchanged.
//   single - one tile per candidate over the whole map: the hat holds every
//            tile; the source tile and both forced-metal port neighbours are
//            skipped, as is the last tried entry. Random initial designs draw
//            one rand_binary() per tile in index order (no mirroring).
//
// Usage:
//   pngf_ref --tiles TX TY --freq F1[,F2...] --gfile PATH [--gfile PATH ...]
//            --seed S [--run-index R] --init empty|random --mode sym|single
//            [--max-evals N] --log OUT
#include <array>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#include <omp.h>

#include "cblas.h"
#include "eigen_subset.hpp"

// The definitions that pngf-opt/main.cpp:58-97 makes before it includes the
// optimizer headers.
typedef double precision;
double operator"" _d(long double v) { return (double)v; }
typedef std::complex<precision> lp_complex;
using namespace std;
using namespace Eigen;

#define eps0 (8.8541878188E-12)
#define mu0 (1.25663706127E-6)
#define c0 (2.997924579998211E8)
#define eta0 (3.767303134118051e+02)

#include "acmetime.hpp"
#include "linalg.hpp"
#include "pngfopt.hpp"
#include "magichat.hpp"

namespace {

struct Args {
  int tx = 7, ty = 7;
  std::vector<double> freqs;
  std::vector<std::string> gfiles;
  int seed = 1, run_index = 0;
  bool init_random = true;
  bool sym = true;
  long max_evals = 0;
  std::string log;
};

std::vector<double> split_doubles(const char *s) {
  std::vector<double> v;
  std::stringstream ss(s);
  std::string tok;
  while (std::getline(ss, tok, ',')) v.push_back(std::atof(tok.c_str()));
  return v;
}

Args parse(int argc, char **argv) {
  Args a;
  for (int i = 1; i < argc; ++i) {
    std::string k = argv[i];
    auto need = [&](int n) {
      if (i + n >= argc) {
        std::fprintf(stderr, "missing value for %s\n", k.c_str());
        std::exit(2);
      }
    };
    if (k == "--tiles") { need(2); a.tx = std::atoi(argv[++i]); a.ty = std::atoi(argv[++i]); }
    else if (k == "--freq") { need(1); a.freqs = split_doubles(argv[++i]); }
    else if (k == "--gfile") { need(1); a.gfiles.push_back(argv[++i]); }
    else if (k == "--seed") { need(1); a.seed = std::atoi(argv[++i]); }
    else if (k == "--run-index") { need(1); a.run_index = std::atoi(argv[++i]); }
    else if (k == "--init") { need(1); a.init_random = std::strcmp(argv[++i], "random") == 0; }
    else if (k == "--mode") { need(1); a.sym = std::strcmp(argv[++i], "sym") == 0; }
    else if (k == "--max-evals") { need(1); a.max_evals = std::atol(argv[++i]); }
    else if (k == "--log") { need(1); a.log = argv[++i]; }
    else { std::fprintf(stderr, "unknown option %s\n", k.c_str()); std::exit(2); }
  }
  if (a.freqs.empty() || a.freqs.size() != a.gfiles.size()) {
    std::fprintf(stderr, "need one --gfile per --freq\n");
    std::exit(2);
  }
  return a;
}

}  // namespace

int main(int argc, char **argv) {
  Args a = parse(argc, argv);
  const int nf = (int)a.freqs.size();
  const int xsz = a.tx, ysz = a.ty;
  const int max_flip_cnt = a.sym ? 4 : 1;
  const int xobj_cnt = 3;
  const precision dx = 0.01 / 60.0, dy = 0.01 / 60.0, dz = 0.01 / 180.0;  // main.cpp:157-160
  std::vector<precision> k0(nf);
  for (int i = 0; i < nf; ++i) k0[i] = 2.0 * M_PI * a.freqs[i] / c0;

  const int qx = (int)((xsz - 1) * 0.5 + 1), qy = (int)((ysz - 1) * 0.5 + 1);
  const int hat_entries = a.sym ? qx * qy - 1 : xsz * ysz;
  MagicHat hat(a.seed, a.run_index, hat_entries);

  std::vector<int> tile_map(xsz * ysz, 0);
  if (a.init_random) {
    if (a.sym) {  // main.cpp:187-208
      for (int j = 0; j < (ysz - 1) * 0.5 + 1; j++)
        for (int i = 0; i < (xsz - 1) * 0.5 + 1; i++) {
          int st = hat.rand_binary();
          tile_map[i + j * xsz] = st;
          if (i < (xsz - 1) * 0.5) tile_map[((xsz - 1) - i) + j * xsz] = st;
          if (j < (ysz - 1) * 0.5) {
            tile_map[i + ((ysz - 1) - j) * xsz] = st;
            if (i < (xsz - 1) * 0.5) tile_map[((xsz - 1) - i) + ((ysz - 1) - j) * xsz] = st;
          }
        }
    } else {
      for (int i = 0; i < xsz * ysz; ++i) tile_map[i] = hat.rand_binary();
    }
  }
  const int mid_x = (int)((xsz - 1) * 0.5), mid_y = (int)((ysz - 1) * 0.5);
  tile_map[mid_y * xsz + mid_x - 1] = 1;  // main.cpp:215-219
  tile_map[mid_y * xsz + mid_x + 1] = 1;
  tile_map[mid_y * xsz + mid_x] = 0;
  tile_map[(mid_y - 1) * xsz + mid_x] = 0;
  tile_map[(mid_y + 1) * xsz + mid_x] = 0;

  std::vector<PNGF_Optimizer> opt(nf);
  acmetime timer;
  timer.tik();
  for (int i = 0; i < nf; ++i) {  // main.cpp:232-253
    opt[i].init(a.gfiles[i].c_str(), xsz, ysz, 3, 3, xobj_cnt, max_flip_cnt, dx, dy, dz);
    opt[i].set_tile_map(tile_map);
    opt[i].set_source_port(mid_x, mid_y, 1, 2);
    opt[i].compute_C_matrix();
    LinAlg::invertMatrix(opt[i].C);
    opt[i].compute_PEinc();
    opt[i].compute_R_matrix(1);
  }
  const double t_init = timer.tok();

  // Objective at one frequency from an Eobj vector (main.cpp:277-289, 407-413).
  auto objective = [&](int ii, const Eigen::Matrix<std::complex<precision>, Dynamic, 1> &eo,
                       std::complex<precision> &S11, precision &D) {
    PNGF_Optimizer &p = opt[ii];
    std::complex<precision> Zin = -(eo(0) + p.Vinc) * dx * 0.5_d / (2.0_d * dy * dz);
    S11 = (Zin - 50.0_d) / (Zin + 50.0_d);
    D = (k0[ii] * k0[ii] / (32 * M_PI * M_PI * eta0)) *
        real(conj(eo(1) + p.LN1inc) * (eo(1) + p.LN1inc) + conj(eo(2) + p.LN2inc) * (eo(2) + p.LN2inc));
    D = 4.0 * M_PI * D / real(-(eo(0) + p.Vinc) * dx * 0.5_d * (2.0_d * dy * dz) * 0.5_d);
    precision m = std::abs(S11);
    return 200.0_d * m * m + (15.0_d - D) * (15.0_d - D);
  };

  std::FILE *log = std::fopen(a.log.c_str(), "w");
  if (!log) {
    std::perror("log");
    return 1;
  }
  std::fprintf(log, "# pngf_ref tiles %d %d nfreq %d seed %d mode %s init %s\n", xsz, ysz, nf,
               a.seed, a.sym ? "sym" : "single", a.init_random ? "random" : "empty");
  std::fprintf(log, "init_map ");
  for (int v : tile_map) std::fputc(v ? 'x' : '.', log);
  std::fputc('\n', log);

  double F_best = 0.0;
  std::vector<std::complex<precision>> s11(nf);
  std::vector<precision> dd(nf);
  for (int ii = 0; ii < nf; ++ii) F_best += objective(ii, opt[ii].Eobj, s11[ii], dd[ii]);
  std::fprintf(log, "start %.17g", F_best);
  for (int ii = 0; ii < nf; ++ii)
    std::fprintf(log, " %.17g %.17g %.17g", s11[ii].real(), s11[ii].imag(), dd[ii]);
  std::fputc('\n', log);

  int last_tried = -1;
  long flip_count = 0, accepts = 0;
  int tile_flip[4], num_flip = 0;
  bool converged = false;
  timer.tik();
  while (true) {
    if (a.max_evals > 0 && flip_count >= a.max_evals) break;
    int tx = 0, ty = 0, rand_tile;
    bool done = false;
    while (true) {  // main.cpp:343-392 (sym) or the single-tile restatement
      rand_tile = hat.draw();
      if (rand_tile < 0) { done = true; break; }
      if (a.sym) {
        ty = rand_tile / qx;
        tx = rand_tile - ty * qx;
      } else {
        ty = rand_tile / xsz;
        tx = rand_tile - ty * xsz;
      }
      if (rand_tile == last_tried) continue;
      if (tx == mid_x && ty == mid_y) continue;
      if (tx == mid_x - 1 && ty == mid_y) continue;
      if (!a.sym && tx == mid_x + 1 && ty == mid_y) continue;
      last_tried = rand_tile;
      if (!a.sym) {
        num_flip = 1;
        tile_flip[0] = tx + ty * xsz;
      } else if (tx == mid_x) {
        num_flip = 2;
        tile_flip[0] = tx + ty * xsz;
        tile_flip[1] = tx + ((ysz - 1) - ty) * xsz;
      } else if (ty == mid_y) {
        num_flip = 2;
        tile_flip[0] = tx + ty * xsz;
        tile_flip[1] = ((xsz - 1) - tx) + ty * xsz;
      } else {
        num_flip = 4;
        tile_flip[0] = tx + ty * xsz;
        tile_flip[1] = ((xsz - 1) - tx) + ty * xsz;
        tile_flip[2] = tx + ((ysz - 1) - ty) * xsz;
        tile_flip[3] = ((xsz - 1) - tx) + ((ysz - 1) - ty) * xsz;
      }
      break;
    }
    if (done) { converged = true; break; }

    double F = 0.0;
    for (int ii = 0; ii < nf; ++ii) {
      opt[ii].compute_updated_Eobj(tile_flip, num_flip);
      F += objective(ii, opt[ii].newEobj, s11[ii], dd[ii]);
    }
    const int accept = F < F_best;
    std::fprintf(log, "eval %ld %d %d %.17g %.17g", flip_count, tx + ty * xsz, accept, F, F_best);
    for (int ii = 0; ii < nf; ++ii)
      std::fprintf(log, " %.17g %.17g %.17g", s11[ii].real(), s11[ii].imag(), dd[ii]);
    std::fputc('\n', log);
    if (accept) {  // main.cpp:429-456
      F_best = F;
      for (int ii = 0; ii < nf; ++ii) {
        opt[ii].update_C_inv();
        opt[ii].compute_PEinc();
        opt[ii].compute_R_matrix(0);
      }
      hat.reset();
      ++accepts;
    }
    ++flip_count;
  }
  const double t_loop = timer.tok();
  std::fprintf(log, "final_map ");
  for (int v : opt[0].tile_map) std::fputc(v ? 'x' : '.', log);
  std::fputc('\n', log);
  std::fprintf(log, "end evals %ld accepts %ld converged %d F %.17g t_init %.6f t_loop %.6f threads %d\n",
               flip_count, accepts, converged ? 1 : 0, F_best, t_init, t_loop, omp_get_max_threads());
  std::fclose(log);
  std::printf("evals %ld accepts %ld converged %d F %.17g t_init %.3f t_loop %.3f\n", flip_count,
              accepts, converged ? 1 : 0, F_best, t_init, t_loop);
  return 0;
}
