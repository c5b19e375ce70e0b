// Host check of colour_wave (units.cuh), the build-time order of the batched
// k-wide products' gathers: on seeded waves of 8 lanes x 8 entries (random
// bank groups, the 8 consecutive rows of a ray's segment, and skewed groups)
// every lane's rounds are a permutation of 0..7 and every bank group with d
// entries in the wave is used at most ceil(d / 8) times a round.  Prints
// "ok <waves>" or the first violation, and exits non-zero on one.
#include <cstdio>
#include <random>

#include "units.cuh"

int main() {
  std::mt19937 rng(12345);
  const int waves = 60000;
  for (int trial = 0; trial < waves; ++trial) {
    unsigned char g[8][8], rd[8][8];
    const int kind = trial % 3;
    for (int j = 0; j < 8; ++j) {
      const int first = (int)(rng() % 8);
      for (int w = 0; w < 8; ++w)
        g[j][w] = (unsigned char)(kind == 0 ? rng() % 8 : kind == 1 ? (first + w) % 8 : rng() % 3);
    }
    if (!plsqr::colour_wave(g, rd)) {
      printf("wave %d: no colouring\n", trial);
      return 1;
    }
    int d[8] = {0};
    for (int j = 0; j < 8; ++j) {
      int seen = 0;
      for (int w = 0; w < 8; ++w) {
        seen |= 1 << rd[j][w];
        ++d[g[j][w]];
      }
      if (seen != 0xff) {
        printf("wave %d: lane %d's rounds are not a permutation\n", trial, j);
        return 1;
      }
    }
    for (int c = 0; c < 8; ++c) {
      int cnt[8] = {0};
      for (int j = 0; j < 8; ++j)
        for (int w = 0; w < 8; ++w)
          if (rd[j][w] == c) ++cnt[g[j][w]];
      for (int q = 0; q < 8; ++q)
        if (cnt[q] > (d[q] + 7) / 8) {
          printf("wave %d: group %d used %d times in round %d (%d entries)\n", trial, q, cnt[q], c,
                 d[q]);
          return 1;
        }
    }
  }
  printf("ok %d\n", waves);
  return 0;
}
