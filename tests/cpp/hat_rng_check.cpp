// Checks the restated MagicHat stream (pngf_gb300/csrc/hat_rng.h) against
// std::mt19937 and std::uniform_int_distribution<int> of the C++ library this
// is built with: raw engine words, bounded draws over many ranges, and whole
// hat passes with swap-removal. Prints "ok" and exits 0 when they agree.
#include <cstdio>
#include <random>
#include <vector>

#include "hat_rng.h"

int main() {
  long checked = 0;
  for (uint32_t seed : {1u, 2u, 5489u, 12345u, 4000000000u}) {
    std::mt19937 ref(seed);
    pngf::MtState m;
    pngf::mt_seed(&m, seed);
    for (int i = 0; i < 5000; ++i, ++checked)
      if (ref() != pngf::mt_next(&m)) {
        std::printf("engine mismatch: seed %u word %d\n", seed, i);
        return 1;
      }
  }
  // bounded draws over ranges small, large and near powers of two
  std::mt19937 ref(7);
  pngf::MtState m;
  pngf::mt_seed(&m, 7);
  std::uniform_int_distribution<> dis;
  const uint32_t ranges[] = {1, 2, 3, 5, 7, 48, 120, 441, 1024, 1025, 1681, 65535, 65536, 65537,
                             1u << 30, (1u << 31) - 1, 2147483647u};
  int used = 0;
  for (int rep = 0; rep < 200; ++rep)
    for (uint32_t r : ranges) {
      dis.param(std::uniform_int_distribution<int>::param_type(0, (int)(r - 1)));
      const int a = dis(ref);
      const int b = (int)pngf::mt_below(&m, r, &used);
      ++checked;
      if (a != b) {
        std::printf("bounded draw mismatch: range %u rep %d: %d vs %d\n", r, rep, a, b);
        return 1;
      }
    }
  // whole hat passes, as MagicHat draws them
  for (int entries : {1, 15, 441, 961}) {
    std::mt19937 g(3);
    std::uniform_int_distribution<> d(0, entries - 1);
    std::vector<int> e1(entries), e2(entries);
    pngf::MtState hm;
    pngf::mt_seed(&hm, 3);
    for (int pass = 0; pass < 3; ++pass) {
      for (int i = 0; i < entries; ++i) e1[i] = e2[i] = i;
      int left1 = entries, left2 = entries;
      while (left1 > 0) {
        d.param(std::uniform_int_distribution<int>::param_type(0, left1 - 1));
        const int idx = d(g);
        const int v1 = e1[idx];
        e1[idx] = e1[left1 - 1];
        --left1;
        const int v2 = pngf::hat_draw(&hm, e2.data(), &left2, &used);
        ++checked;
        if (v1 != v2 || left1 != left2) {
          std::printf("hat mismatch: entries %d pass %d\n", entries, pass);
          return 1;
        }
      }
      if (pngf::hat_draw(&hm, e2.data(), &left2, &used) != -1) return 1;
    }
  }
  std::printf("ok %ld\n", checked);
  return 0;
}
