// A pngf-opt/main.cpp-style DBS program written against the drop-in class
// include/pngf_optimizer.hpp (one PNGF_Optimizer per frequency, the same
// call sequence as main.cpp:232-253, 402-452). Used by the GPU tests to show
// that code written for the reference class runs unchanged on the library and
// reproduces the reference's golden logs.
//
// Usage: dropin_main --tiles TX TY --freq F1[,F2..] --gfile P [--gfile P ..]
//                    --seed S --init empty|random --mode sym|single --log OUT
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#include "pngf_optimizer.hpp"

typedef double precision;
static const double c0 = 2.997924579998211E8, eta0 = 3.767303134118051e+02;

// Draw-without-replacement hat with the standard engine and distribution
// that pngf-opt/magichat.hpp uses.
struct Hat {
  std::mt19937 gen;
  std::uniform_int_distribution<> dis;
  int total, left;
  std::vector<int> e;
  Hat(int seed, int n) : total(n), left(n), e(n) {
    gen.seed(seed);
    dis = std::uniform_int_distribution<>(0, n - 1);
    for (int i = 0; i < n; ++i) e[i] = i;
  }
  int rand_binary() { return gen() & 1; }
  int draw() {
    if (left <= 0) return -1;
    dis.param(std::uniform_int_distribution<int>::param_type(0, left - 1));
    int idx = dis(gen), v = e[idx];
    e[idx] = e[left - 1];
    --left;
    return v;
  }
  void reset() {
    for (int i = 0; i < total; ++i) e[i] = i;
    left = total;
  }
};

int main(int argc, char **argv) {
  int xsz = 7, ysz = 7, seed = 1;
  bool init_random = true, sym = true;
  std::vector<double> freqs;
  std::vector<std::string> gfiles;
  std::string logp;
  for (int i = 1; i < argc; ++i) {
    std::string k = argv[i];
    if (k == "--tiles") { xsz = std::atoi(argv[++i]); ysz = std::atoi(argv[++i]); }
    else if (k == "--freq") {
      std::stringstream ss(argv[++i]);
      std::string t;
      while (std::getline(ss, t, ',')) freqs.push_back(std::atof(t.c_str()));
    } else if (k == "--gfile") gfiles.push_back(argv[++i]);
    else if (k == "--seed") seed = std::atoi(argv[++i]);
    else if (k == "--init") init_random = std::strcmp(argv[++i], "random") == 0;
    else if (k == "--mode") sym = std::strcmp(argv[++i], "sym") == 0;
    else if (k == "--log") logp = argv[++i];
  }
  const int NUM_FREQ = (int)freqs.size();
  const precision dx = 0.01 / 60.0, dy = 0.01 / 60.0, dz = 0.01 / 180.0;
  const int qx = (int)((xsz - 1) * 0.5 + 1), qy = (int)((ysz - 1) * 0.5 + 1);
  Hat hat(seed, sym ? qx * qy - 1 : xsz * ysz);
  std::vector<int> tile_map(xsz * ysz, 0);
  if (init_random) {
    if (sym) {
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
  const int mx = (int)((xsz - 1) * 0.5), my = (int)((ysz - 1) * 0.5);
  tile_map[my * xsz + mx - 1] = 1;
  tile_map[my * xsz + mx + 1] = 1;
  tile_map[my * xsz + mx] = 0;
  tile_map[(my - 1) * xsz + mx] = 0;
  tile_map[(my + 1) * xsz + mx] = 0;

  // The reference's per-frequency setup sequence (main.cpp:232-253).
  std::vector<PNGF_Optimizer> myPNGF(NUM_FREQ);
  for (int i = 0; i < NUM_FREQ; i++) {
    myPNGF[i].init(gfiles[i].c_str(), xsz, ysz, 3, 3, 3, sym ? 4 : 1, dx, dy, dz);
    myPNGF[i].set_tile_map(tile_map);
    myPNGF[i].set_source_port(mx, my, 1, 2);
    myPNGF[i].compute_C_matrix();
    LinAlg::invertMatrix(myPNGF[i].C);
    myPNGF[i].compute_PEinc();
    myPNGF[i].compute_R_matrix(1);
  }
  std::vector<precision> k0(NUM_FREQ);
  for (int i = 0; i < NUM_FREQ; i++) k0[i] = 2.0 * M_PI * freqs[i] / c0;
  auto term = [&](int ii, PNGF_Optimizer::CVec &eo, std::complex<double> &S11, double &D) {
    PNGF_Optimizer &p = myPNGF[ii];
    std::complex<double> Zin = -(eo(0) + p.Vinc) * dx * 0.5 / (2.0 * dy * dz);
    S11 = (Zin - 50.0) / (Zin + 50.0);
    D = (k0[ii] * k0[ii] / (32 * M_PI * M_PI * eta0)) *
        real(conj(eo(1) + p.LN1inc) * (eo(1) + p.LN1inc) + conj(eo(2) + p.LN2inc) * (eo(2) + p.LN2inc));
    D = 4.0 * M_PI * D / real(-(eo(0) + p.Vinc) * dx * 0.5 * (2.0 * dy * dz) * 0.5);
    double m = std::abs(S11);
    return 200.0 * m * m + (15.0 - D) * (15.0 - D);
  };
  FILE *log = std::fopen(logp.c_str(), "w");
  std::fprintf(log, "init_map ");
  for (int v : tile_map) std::fputc(v ? 'x' : '.', log);
  std::fputc('\n', log);
  double F_best = 0.0;
  std::vector<std::complex<double>> s11(NUM_FREQ);
  std::vector<double> dd(NUM_FREQ);
  for (int ii = 0; ii < NUM_FREQ; ++ii) F_best += term(ii, myPNGF[ii].Eobj, s11[ii], dd[ii]);
  std::fprintf(log, "start %.17g\n", F_best);
  int last_tried = -1, tile_flip[4], num_flip = 0;
  long flip_count = 0;
  while (true) {  // main.cpp:338-459
    int tx = 0, ty = 0, r;
    bool done = false;
    while (true) {
      r = hat.draw();
      if (r < 0) { done = true; break; }
      if (sym) { ty = r / qx; tx = r - ty * qx; } else { ty = r / xsz; tx = r - ty * xsz; }
      if (r == last_tried) continue;
      if (tx == mx && ty == my) continue;
      if (tx == mx - 1 && ty == my) continue;
      if (!sym && tx == mx + 1 && ty == my) continue;
      last_tried = r;
      if (!sym) { num_flip = 1; tile_flip[0] = tx + ty * xsz; }
      else if (tx == mx) { num_flip = 2; tile_flip[0] = tx + ty * xsz; tile_flip[1] = tx + ((ysz - 1) - ty) * xsz; }
      else if (ty == my) { num_flip = 2; tile_flip[0] = tx + ty * xsz; tile_flip[1] = ((xsz - 1) - tx) + ty * xsz; }
      else {
        num_flip = 4;
        tile_flip[0] = tx + ty * xsz;
        tile_flip[1] = ((xsz - 1) - tx) + ty * xsz;
        tile_flip[2] = tx + ((ysz - 1) - ty) * xsz;
        tile_flip[3] = ((xsz - 1) - tx) + ((ysz - 1) - ty) * xsz;
      }
      break;
    }
    if (done) break;
    double F = 0.0;
    for (int ii = 0; ii < NUM_FREQ; ii++) {
      myPNGF[ii].compute_updated_Eobj(tile_flip, num_flip);
      F += term(ii, myPNGF[ii].newEobj, s11[ii], dd[ii]);
    }
    const int acc = F < F_best;
    std::fprintf(log, "eval %ld %d %d %.17g %.17g", flip_count, tx + ty * xsz, acc, F, F_best);
    for (int ii = 0; ii < NUM_FREQ; ++ii) std::fprintf(log, " %.17g %.17g %.17g", s11[ii].real(), s11[ii].imag(), dd[ii]);
    std::fputc('\n', log);
    if (acc) {
      F_best = F;
      for (int ii = 0; ii < NUM_FREQ; ii++) {
        myPNGF[ii].update_C_inv();
        myPNGF[ii].compute_PEinc();
        myPNGF[ii].compute_R_matrix(0);
      }
      hat.reset();
    }
    flip_count++;
  }
  std::fprintf(log, "final_map ");
  for (int v : myPNGF[0].tile_map) std::fputc(v ? 'x' : '.', log);
  std::fputc('\n', log);
  std::fprintf(log, "end evals %ld converged 1 F %.17g\n", flip_count, F_best);
  std::fclose(log);
  return 0;
}
