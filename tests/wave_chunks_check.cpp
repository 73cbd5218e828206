// Host check of wave_chunks (clk_internal.h), the z-chunk count for kernels
// whose CTAs each stream one tile through a z-chunk: the counts it picks for
// the measured cases, and that the chosen count never costs more waves x
// planes than one chunk per tile.  Built and run by tests/test_wave_chunks.py.
#include <cstdio>

#include "clk_internal.h"

static int g_fail = 0;
static void expect(const char* what, int got, int want) {
  if (got != want) {
    std::printf("FAIL %s: %d, want %d\n", what, got, want);
    g_fail = 1;
  }
}

static double cost(long long tiles, int depth, int halo, long long slots, int c) {
  const int zc = (depth + c - 1) / c, n = (depth + zc - 1) / zc;
  return (double)((tiles * n + slots - 1) / slots) * (zc + halo);
}

int main() {
  // sobel_3d on 1024x1024x256 (16x64 tiles, 3 halo planes): 2 CTAs per SM
  // leave a last wave of 112 CTAs with one chunk per tile; two chunks fill it
  expect("sobel, 2 CTAs per SM", clk::wave_chunks(1024, 256, 3, 152 * 2, 1, 16), 2);
  // the 256x256x64 Gaussian (4x8 tiles, 2cz = 6): eight chunks of 8 planes
  // fill 256 of the 304 slots in one wave
  expect("small Gaussian", clk::wave_chunks(32, 64, 6, 152 * 2, 1, 16), 8);
  // z pairs: chunks of whole pairs
  expect("pairs", clk::wave_chunks(2048, 256, 4, 152 * 2, 2, 16), 1);
  for (long long tiles : {1LL, 7LL, 32LL, 152LL, 500LL, 1024LL, 4096LL})
    for (int depth : {1, 2, 3, 17, 64, 255, 400})
      for (int halo : {0, 2, 6, 10})
        for (long long slots : {152LL, 304LL, 608LL}) {
          const int c = clk::wave_chunks(tiles, depth, halo, slots, 1, 16);
          if (c < 1 || c > 16 || cost(tiles, depth, halo, slots, c) > cost(tiles, depth, halo, slots, 1)) {
            std::printf("FAIL tiles %lld depth %d halo %d slots %lld: %d\n", tiles, depth, halo, slots, c);
            g_fail = 1;
          }
        }
  if (g_fail) return 1;
  std::printf("ok\n");
  return 0;
}
