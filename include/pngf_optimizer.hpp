// Drop-in replacement for the reference's optimizer class, over the C ABI.
//
// pngf-opt/main.cpp drives one PNGF_Optimizer per frequency
// (main.cpp:166, 224-253, 406, 447-452) and reads its public members
// Eobj, newEobj, Vinc, LN1inc, LN2inc and tile_map (main.cpp:277-284,
// 407-411, 314, 481). This header provides a class of the same name with the
// same methods and members, backed by a single-frequency pngf_handle on the
// GPU, plus LinAlg::invertMatrix for its C member, so main.cpp compiles
// against it after replacing
//     #include "linalg.hpp"
//     #include "pngfopt.hpp"
// with
//     #include "pngf_optimizer.hpp"
// and linking -lpngf_gb300. Errors that the reference prints and ignores
// (missing G file, pngfopt.hpp:122-127) are printed the same way here.
//
// Replaces pngf-opt/pngfopt.hpp:18-679 and pngf-opt/linalg.hpp:18-85.
#pragma once

#include <complex>
#include <cstdio>
#include <vector>

#include "pngf_gb300.h"

class PNGF_Optimizer {
 public:
  // Column vector with Eigen-style element access, e.g. Eobj(0).
  struct CVec {
    std::vector<std::complex<double>> v;
    std::complex<double> &operator()(int i) { return v[i]; }
    const std::complex<double> &operator()(int i) const { return v[i]; }
    long rows() const { return (long)v.size(); }
  };
  // Stand-in for the C member: the GPU keeps M = [[H C^-1, y], [R, Eobj]]
  // instead of C^-1, so inversion happens inside compute_R_matrix(1).
  struct CMatrix {
    PNGF_Optimizer *owner = nullptr;
  };

  CVec Eobj, newEobj;
  std::complex<double> Vinc, LN1inc, LN2inc;
  std::vector<int> tile_map;
  CMatrix C;
  int map_xsz = 0, map_ysz = 0, map_sz = 0, num_eobj = 0;

  PNGF_Optimizer() { C.owner = this; }
  PNGF_Optimizer(const PNGF_Optimizer &) = delete;
  PNGF_Optimizer &operator=(const PNGF_Optimizer &) = delete;
  PNGF_Optimizer(PNGF_Optimizer &&o) noexcept { *this = static_cast<PNGF_Optimizer &&>(o); }
  PNGF_Optimizer &operator=(PNGF_Optimizer &&o) noexcept {
    std::swap(h_, o.h_);
    Eobj = o.Eobj;
    newEobj = o.newEobj;
    Vinc = o.Vinc;
    LN1inc = o.LN1inc;
    LN2inc = o.LN2inc;
    tile_map = o.tile_map;
    map_xsz = o.map_xsz;
    map_ysz = o.map_ysz;
    map_sz = o.map_sz;
    num_eobj = o.num_eobj;
    max_flips_ = o.max_flips_;
    last_ = o.last_;
    C.owner = this;
    return *this;
  }
  ~PNGF_Optimizer() {
    if (h_) pngf_destroy(h_);
  }

  // pngfopt.hpp:66-191
  void init(const char *filename, int num_tiles_x, int num_tiles_y, int num_cells_per_tile_x,
            int num_cells_per_tile_y, int tnum_eobj, int max_flips, double mdx, double mdy, double mdz) {
    pngf_config cfg;
    pngf_config_default(&cfg, num_tiles_x, num_tiles_y, 1, nullptr);
    cfg.cells_x = num_cells_per_tile_x;
    cfg.cells_y = num_cells_per_tile_y;
    cfg.num_eobj = tnum_eobj;
    cfg.max_flips = max_flips;
    cfg.dx = mdx;
    cfg.dy = mdy;
    cfg.dz = mdz;
    if (h_) pngf_destroy(h_);
    h_ = nullptr;
    int rc = pngf_create(&cfg, &h_);
    if (rc != PNGF_OK) {
      std::printf("pngf_create failed: %d\n", rc);
      return;
    }
    map_xsz = num_tiles_x;
    map_ysz = num_tiles_y;
    map_sz = map_xsz * map_ysz;
    num_eobj = tnum_eobj;
    max_flips_ = max_flips;
    tile_map.assign(map_sz, 0);
    Eobj.v.assign(num_eobj, 0.0);
    newEobj.v.assign(num_eobj, 0.0);
    if (pngf_load_G_file(h_, 0, filename) != PNGF_OK) std::printf("Error file %s not found!\n", filename);
  }

  // pngfopt.hpp:669-674
  void set_tile_map(std::vector<int> &input_map) {
    tile_map = input_map;
    check(pngf_set_tile_map(h_, tile_map.data()), "set_tile_map");
  }
  // pngfopt.hpp:559-618
  void set_source_port(int port_tile_x, int port_tile_y, int port_y_offset, int port_y_size) {
    check(pngf_set_source_port(h_, port_tile_x, port_tile_y, port_y_offset, port_y_size), "set_source_port");
  }
  // pngfopt.hpp:196-233 and 542-552: folded into compute_R_matrix(1).
  void compute_C_matrix() {}
  void compute_PEinc() {}
  // pngfopt.hpp:237-250
  void compute_R_matrix(int compute_eobj) {
    if (compute_eobj) {
      check(pngf_prepare(h_), "prepare");
      read_eobj(Eobj);
      newEobj = Eobj;
    } else {
      Eobj = newEobj;
    }
  }
  // pngfopt.hpp:379-539
  std::complex<double> compute_updated_Eobj(int *tile_idx, int num_tiles_to_flip) {
    std::vector<int> tiles(max_flips_, 0);
    for (int i = 0; i < num_tiles_to_flip && i < max_flips_; ++i) tiles[i] = tile_idx[i];
    int nflip = num_tiles_to_flip;
    std::vector<double> eo(2 * num_eobj);
    check(pngf_eval_candidates(h_, tiles.data(), &nflip, 1, eo.data(), nullptr), "compute_updated_Eobj");
    for (int e = 0; e < num_eobj; ++e) newEobj.v[e] = {eo[2 * e], eo[2 * e + 1]};
    last_.assign(tile_idx, tile_idx + num_tiles_to_flip);
    return newEobj(0);
  }
  // pngfopt.hpp:256-367
  void update_C_inv() {
    if (check(pngf_accept(h_, 0), "update_C_inv") == PNGF_OK)
      for (int t : last_) tile_map[t] ^= 1;
  }

  pngf_handle *handle() { return h_; }

 private:
  pngf_handle *h_ = nullptr;
  int max_flips_ = 1;
  std::vector<int> last_;

  int check(int rc, const char *what) {
    if (rc != PNGF_OK) std::printf("%s: %s\n", what, pngf_last_error(h_));
    return rc;
  }
  void read_eobj(CVec &out) {
    std::vector<double> eo(2 * num_eobj), vl(6);
    check(pngf_get_eobj(h_, 0, eo.data(), vl.data()), "get_eobj");
    for (int e = 0; e < num_eobj; ++e) out.v[e] = {eo[2 * e], eo[2 * e + 1]};
    Vinc = {vl[0], vl[1]};
    LN1inc = {vl[2], vl[3]};
    LN2inc = {vl[4], vl[5]};
  }
};

// linalg.hpp:34-85. The inverse is formed inside compute_R_matrix(1).
class LinAlg {
 public:
  static int invertMatrix(PNGF_Optimizer::CMatrix &) { return 1; }
};
