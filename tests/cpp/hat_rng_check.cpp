// Checks the restated MagicHat stream (pngf_gb300/csrc/hat_rng.h) against
// std::mt19937 and std::uniform_int_distribution<int> of the C++ library this
// is built with: raw engine words, bounded draws over many ranges, and whole
// hat passes with swap-removal. Prints "ok" and exits 0 when they agree.
#include <cstdio>
#include <cstdlib>
#include <random>
#include <string>
#include <vector>

#include "hat_rng.h"

// Sequence mode: the candidate order of a DBS run whose accept decisions
// follow a fixed rule (evaluated candidate n is accepted when n % 7 == 3),
// drawn two ways -- one candidate at a time, as the reference does, and in
// speculative batches of B replayed as the device loop does (engine restored
// to the batch start and advanced by the outputs the draws up to the accepted
// one consumed; last_tried = that draw's hat value; the hat refilled). Both
// must agree; the reference-order sequence is printed for comparison with the
// oracle: one line "log_index t0 t1 .." per evaluated candidate.
static int sequence_mode(int tx, int ty, int sym, unsigned seed, int binary_draws, int B, int evals) {
  const int qx = (int)((tx - 1) * 0.5 + 1), qy = (int)((ty - 1) * 0.5 + 1);
  const int entries = sym ? qx * qy - 1 : tx * ty;
  const pngf::HatGeom g{tx, ty, qx, (int)((tx - 1) * 0.5), (int)((ty - 1) * 0.5), sym};
  auto accept_rule = [](long n) { return n % 7 == 3; };
  struct Cand {
    int li, nf, t[4];
  };
  // one at a time
  std::vector<Cand> seq;
  {
    pngf::MtState m;
    pngf::mt_seed(&m, seed);
    for (int i = 0; i < binary_draws; ++i) pngf::mt_next(&m);
    std::vector<int> ent(entries);
    for (int i = 0; i < entries; ++i) ent[i] = i;
    int left = entries, last = -1, used = 0;
    while ((int)seq.size() < evals) {
      Cand c{};
      const int r = pngf::hat_draw(&m, ent.data(), &left, &used);
      if (r < 0) break;  // hat empty: converged
      if (!pngf::hat_candidate(g, r, &last, &c.li, &c.nf, c.t)) continue;
      seq.push_back(c);
      if (accept_rule((long)seq.size() - 1)) {
        for (int i = 0; i < entries; ++i) ent[i] = i;
        left = entries;
      }
    }
  }
  // speculative batches with replay
  std::vector<Cand> spec;
  {
    pngf::MtState m;
    pngf::mt_seed(&m, seed);
    for (int i = 0; i < binary_draws; ++i) pngf::mt_next(&m);
    std::vector<int> ent(entries);
    for (int i = 0; i < entries; ++i) ent[i] = i;
    int left = entries, last = -1;
    while ((int)spec.size() < evals) {
      const pngf::MtState m0 = m;
      std::vector<Cand> batch;
      std::vector<int> used_at, r_at;
      int used = 0;
      bool empty = false;
      while ((int)batch.size() < B) {
        Cand c{};
        const int r = pngf::hat_draw(&m, ent.data(), &left, &used);
        if (r < 0) {
          empty = true;
          break;
        }
        if (!pngf::hat_candidate(g, r, &last, &c.li, &c.nf, c.t)) continue;
        batch.push_back(c);
        used_at.push_back(used);
        r_at.push_back(r);
      }
      int j = -1;
      for (int i = 0; i < (int)batch.size() && j < 0; ++i)
        if (accept_rule((long)spec.size() + i)) j = i;
      const int take = j >= 0 ? j + 1 : (int)batch.size();
      for (int i = 0; i < take && (int)spec.size() < evals; ++i) spec.push_back(batch[i]);
      if (j >= 0) {
        m = m0;
        for (int q = 0; q < used_at[j]; ++q) pngf::mt_next(&m);
        last = r_at[j];
        for (int i = 0; i < entries; ++i) ent[i] = i;
        left = entries;
      } else if (empty || batch.empty()) {
        break;
      }
    }
  }
  if (seq.size() != spec.size()) {
    std::printf("length mismatch %zu vs %zu\n", seq.size(), spec.size());
    return 1;
  }
  for (size_t i = 0; i < seq.size(); ++i) {
    if (seq[i].li != spec[i].li || seq[i].nf != spec[i].nf) {
      std::printf("replay mismatch at %zu\n", i);
      return 1;
    }
    std::printf("%d", seq[i].li);
    for (int q = 0; q < seq[i].nf; ++q) std::printf(" %d", seq[i].t[q]);
    std::printf("\n");
  }
  return 0;
}

int main(int argc, char **argv) {
  if (argc == 9 && std::string(argv[1]) == "seq")
    return sequence_mode(std::atoi(argv[2]), std::atoi(argv[3]), std::atoi(argv[4]), (unsigned)std::atol(argv[5]),
                         std::atoi(argv[6]), std::atoi(argv[7]), std::atoi(argv[8]));
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
