// MagicHat's random stream restated for the device (pngf-opt/magichat.hpp:53-107).
//
// MagicHat draws with std::mt19937 and std::uniform_int_distribution<int>.
// The device-resident DBS loop needs the same stream without the C++
// library, so this header restates both as plain functions usable on the host
// and on the device:
//
//  * MT19937, M. Matsumoto and T. Nishimura, "Mersenne Twister: a
//    623-dimensionally equidistributed uniform pseudo-random number
//    generator", ACM TOMACS 8(1), 1998 (the parameters are the ones the C++
//    standard fixes for std::mt19937, [rand.predef]);
//  * the bounded integer of GCC's libstdc++ (since GCC 11) for a 32-bit
//    engine: D. Lemire, "Fast Random Integer Generation in an Interval", ACM
//    TOMACS 29(1), 2019 -- multiply-shift with a rejection threshold.
//
// The second depends on the C++ library the host driver was built with, so
// the device loop checks these functions against the library's own engine and
// distribution before it runs (hat_rng_matches_std in dbs.cpp) and refuses to
// start when they differ.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define PNGF_HD __host__ __device__ __forceinline__
#else
#define PNGF_HD inline
#endif

namespace pngf {

constexpr int kMtN = 624, kMtM = 397;

struct MtState {
  uint32_t x[kMtN];
  int i;  // next word of x to temper; kMtN = regenerate first
};

PNGF_HD void mt_seed(MtState *m, uint32_t s) {
  m->x[0] = s;
  for (int i = 1; i < kMtN; ++i) m->x[i] = 1812433253u * (m->x[i - 1] ^ (m->x[i - 1] >> 30)) + (uint32_t)i;
  m->i = kMtN;
}

PNGF_HD uint32_t mt_mix(uint32_t a, uint32_t b, uint32_t c) {
  const uint32_t y = (a & 0x80000000u) | (b & 0x7fffffffu);
  return c ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
}

PNGF_HD void mt_regenerate(MtState *m) {
  uint32_t *x = m->x;
  int k = 0;
  for (; k < kMtN - kMtM; ++k) x[k] = mt_mix(x[k], x[k + 1], x[k + kMtM]);
  for (; k < kMtN - 1; ++k) x[k] = mt_mix(x[k], x[k + 1], x[k + kMtM - kMtN]);
  x[kMtN - 1] = mt_mix(x[kMtN - 1], x[0], x[kMtM - 1]);
  m->i = 0;
}

PNGF_HD uint32_t mt_next(MtState *m) {
  if (m->i >= kMtN) mt_regenerate(m);
  uint32_t y = m->x[m->i++];
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}

// Uniform integer in [0, range), range >= 1; *used counts the engine outputs
// consumed (the device loop replays a hat by that count).
PNGF_HD uint32_t mt_below(MtState *m, uint32_t range, int *used) {
  uint64_t p = (uint64_t)mt_next(m) * range;
  ++*used;
  uint32_t lo = (uint32_t)p;
  if (lo < range) {
    const uint32_t t = (0u - range) % range;
    while (lo < t) {
      p = (uint64_t)mt_next(m) * range;
      ++*used;
      lo = (uint32_t)p;
    }
  }
  return (uint32_t)(p >> 32);
}

// MagicHat::draw (magichat.hpp:84-99): a uniform entry of the remaining ones,
// swap-removed; -1 when the hat is empty.
PNGF_HD int hat_draw(MtState *m, int *entry, int *left, int *used) {
  if (*left <= 0) return -1;
  const int idx = (int)mt_below(m, (uint32_t)*left, used);
  const int val = entry[idx];
  entry[idx] = entry[*left - 1];
  --*left;
  return val;
}

// The candidate of hat value r (main.cpp:343-392): the skip rules, then the
// tiles it flips (its mirror images in the 4-fold symmetric mode). Returns
// false when r is skipped; *last_tried is updated as the reference does.
struct HatGeom {
  int tiles_x, tiles_y, qx, mid_x, mid_y, sym;
};

PNGF_HD bool hat_candidate(const HatGeom &g, int r, int *last_tried, int *log_index, int *nflip, int *tiles) {
  int tx, ty;
  if (g.sym) {
    ty = r / g.qx;
    tx = r - ty * g.qx;
  } else {
    ty = r / g.tiles_x;
    tx = r - ty * g.tiles_x;
  }
  if (r == *last_tried) return false;
  if (tx == g.mid_x && ty == g.mid_y) return false;      // source tile
  if (tx == g.mid_x - 1 && ty == g.mid_y) return false;  // metal next to the source
  if (!g.sym && tx == g.mid_x + 1 && ty == g.mid_y) return false;
  *last_tried = r;
  const int xsz = g.tiles_x, ysz = g.tiles_y;
  *log_index = tx + ty * xsz;
  tiles[0] = tx + ty * xsz;
  if (!g.sym) {
    *nflip = 1;
  } else if (tx == g.mid_x) {
    *nflip = 2;
    tiles[1] = tx + ((ysz - 1) - ty) * xsz;
  } else if (ty == g.mid_y) {
    *nflip = 2;
    tiles[1] = ((xsz - 1) - tx) + ty * xsz;
  } else {
    *nflip = 4;
    tiles[1] = ((xsz - 1) - tx) + ty * xsz;
    tiles[2] = tx + ((ysz - 1) - ty) * xsz;
    tiles[3] = ((xsz - 1) - tx) + ((ysz - 1) - ty) * xsz;
  }
  return true;
}

}  // namespace pngf
