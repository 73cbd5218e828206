"""The generated median networks (clk_median_networks.cuh) compiled for the
host with plain ints, checked on random inputs with the sorted-run
structure each network assumes: every selected rank must equal the rank of
a full sort."""
import subprocess

import pytest

from conftest import ROOT

PROG = r"""
#include <algorithm>
#include <cstdio>
#include <random>
#include <vector>
#define CLK_NET_FN inline
#define CLK_NET_CONST constexpr
static inline int vmin(int a, int b) { return a < b ? a : b; }
static inline int vmax(int a, int b) { return a < b ? b : a; }
#include "clk_median_networks.cuh"
static std::mt19937 rng(7);
static void runs(std::vector<int>& v, std::vector<std::pair<int,int>> r) {
  for (auto [a, b] : r) std::sort(v.begin() + a, v.begin() + b);
}
template <int N, class F> static int check(const char* name, std::vector<std::pair<int,int>> sorted_runs,
                                           const int* outw, int nout, int first_rank, F net, int vmax_) {
  for (int t = 0; t < 200000; ++t) {
    std::vector<int> v(N);
    for (auto& x : v) x = (int)(rng() % vmax_);
    runs(v, sorted_runs);
    std::vector<int> s = v;
    std::sort(s.begin(), s.end());
    int w[N];
    for (int i = 0; i < N; ++i) w[i] = v[i];
    net(w);
    for (int k = 0; k < nout; ++k)
      if (w[outw[k]] != s[first_rank + k]) { std::printf("FAIL %s rank %d\n", name, first_rank + k); return 1; }
  }
  return 0;
}
int main() {
  int bad = 0;
  for (int vm : {2, 5, 1000}) {
    bad |= check<3>("sort3", {}, net_sort3_out, 3, 0, [](int (&w)[3]) { net_sort3_raw(w); }, vm);
    bad |= check<9>("merge333", {{0,3},{3,6},{6,9}}, net_merge333_out, 9, 0, [](int (&w)[9]) { net_merge333_raw(w); }, vm);
    bad |= check<18>("merge99_mid", {{0,9},{9,18}}, net_merge99_mid_out, 10, 4, [](int (&w)[18]) { net_merge99_mid_raw(w); }, vm);
    bad |= check<19>("box27_final", {{0,10},{10,19}}, net_box27_final_out, 1, 9, [](int (&w)[19]) { net_box27_final_raw(w); }, vm);
    bad |= check<33>("sphere33_final", {{0,9},{9,18},{18,27}}, net_sphere33_final_out, 1, 16, [](int (&w)[33]) { net_sphere33_final_raw(w); }, vm);
    bad |= check<9>("med9", {{0,3},{3,6},{6,9}}, net_med9_out, 1, 4, [](int (&w)[9]) { net_med9_raw(w); }, vm);
    bad |= check<18>("merge99_r1_16", {{0,9},{9,18}}, net_merge99_r1_16_out, 16, 1, [](int (&w)[18]) { net_merge99_r1_16_raw(w); }, vm);
    bad |= check<31>("sphere33_pair_final", {{0,16},{16,25}}, net_sphere33_pair_final_out, 1, 15,
                     [](int (&w)[31]) { net_sphere33_pair_final_raw(w); }, vm);
    // the z-pair composition: median of 33 = rank 15 of (ranks 1..16 of the
    // shared planes' merge, the other plane's sorted 9, 6 singles)
    for (int t = 0; t < 200000; ++t) {
      std::vector<int> v(33);
      for (auto& x : v) x = (int)(rng() % vm);
      runs(v, {{0,9},{9,18},{18,27}});
      std::vector<int> s = v;
      std::sort(s.begin(), s.end());
      int m[18];
      for (int i = 0; i < 18; ++i) m[i] = v[i];
      net_merge99_r1_16_raw(m);
      int w[31];
      for (int i = 0; i < 16; ++i) w[i] = m[net_merge99_r1_16_out[i]];
      for (int i = 0; i < 15; ++i) w[16 + i] = v[18 + i];
      net_sphere33_pair_final_raw(w);
      if (w[net_sphere33_pair_final_out[0]] != s[16]) { std::puts("FAIL sphere33 pair composition"); bad = 1; break; }
    }
  }
  std::puts(bad ? "FAILED" : "ok");
  return bad;
}
"""


def test_generated_networks_select_the_right_ranks(tmp_path):
    src = tmp_path / "nets.cpp"
    src.write_text(PROG)
    exe = tmp_path / "nets"
    csrc = ROOT / "clij-opencl-kernels_gb300" / "csrc"
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-I", str(csrc), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    if r.returncode != 0:
        pytest.fail(r.stderr)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "ok" in r.stdout, r.stdout + r.stderr


def test_box27_composition_equals_median():
    """The box kernel's decomposition: median of 27 = rank 9 of (ranks 4..13 of
    merge(P_z, P_z+1)) U P_z-1, where P are the sorted planes' 3x3 blocks."""
    import numpy as np
    rng = np.random.default_rng(0)
    for _ in range(20000):
        v = rng.integers(0, 7, size=27)
        p = [np.sort(v[9 * i:9 * i + 9]) for i in range(3)]
        m = np.sort(np.concatenate([p[1], p[2]]))[4:14]
        got = np.sort(np.concatenate([m, p[0]]))[9]
        assert got == np.sort(v)[13]
