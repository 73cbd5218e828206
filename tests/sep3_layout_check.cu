// Host-side check of the register-ring separable kernels' address
// arithmetic (clk_sep3.cuh): for every instantiated operation, XY radius,
// Z radius and the launch shapes in use, and a range of image extents, it
// recomputes each thread's shared-memory and global offsets exactly as the
// kernel does and checks that every access stays inside its buffer (and,
// for the staged rows, inside its row).  Built and run by
// tests/test_sep3_layout.py on the CPU; prints "ok" and exits 0, or
// reports the first offending access and exits 1.
#include <cstdio>
#include <cstdlib>

#include "clk_sep3.cuh"

namespace clk {
clk_status check_launch(const char*) { return CLK_OK; }
void count_launch(int) {}
}  // namespace clk

using namespace clk;
using namespace clk::sep3;

static int hclamp(int v, int hi) { return v < 0 ? 0 : v > hi ? hi : v; }  // clamp-to-edge index

static long long g_checks = 0;
static int g_fail = 0;

#define REQUIRE(cond, ...)                                                          \
  do {                                                                              \
    ++g_checks;                                                                     \
    if (!(cond)) {                                                                  \
      if (!g_fail) {                                                                \
        std::printf("FAIL %s:%d: ", __FILE__, __LINE__);                            \
        std::printf(__VA_ARGS__);                                                   \
        std::printf("\n");                                                          \
      }                                                                             \
      g_fail = 1;                                                                   \
      return;                                                                       \
    }                                                                               \
  } while (0)

template <int OP, int R, int CZ, class C> void check_cta(int W, int H, int bx, int by) {
  using G = Geo<OP, R, CZ, C>;
  constexpr int NT = C::NT, SEGY = C::SEGY, MX = G::MX, TY = C::TY;
  constexpr size_t RAWTOT = (size_t)G::NRAW * G::RAW_BYTES;
  const int x0 = bx * TX, y0 = by * TY;
  const size_t plane = (size_t)W * H;
  for (int tid = 0; tid < NT; ++tid) {
    // staging
    for (int k = 0; k < G::PST; ++k) {
      const int q = tid + k * NT;
      if (q >= G::NST) continue;
      const int v = q % G::NV, r = q / G::NV;
      const int gx = x0 - G::RA + 8 * v;
      const int ra = OP == GAUSS ? 2 * r : r;
      const bool outside = gx < 0 || gx >= W;
      const size_t goff = (size_t)hclamp(y0 - R + ra, H - 1) * W + (size_t)std::min(std::max(gx, 0), W - 8);
      const size_t soff = (size_t)(ra * G::RWP + 8 * v) * 2;
      REQUIRE(goff + 8 <= plane, "op %d R %d cz %d staging global %zu of %zu", OP, R, CZ, goff + 8, plane);
      REQUIRE(goff % 8 == 0, "staging global offset %zu not 16-byte aligned", goff);
      REQUIRE(soff + 16 <= (size_t)G::RAW_BYTES, "op %d R %d staging smem %zu of %d", OP, R, soff + 16, G::RAW_BYTES);
      REQUIRE(8 * v + 8 <= G::SW, "staging vector past the staged row");
      if (OP == GAUSS) {
        const size_t g2 = (size_t)hclamp(y0 - R + 2 * r + 1, H - 1) * W + (size_t)std::min(std::max(gx, 0), W - 8);
        REQUIRE(g2 + 8 <= plane, "gauss second row global");
        REQUIRE(soff + G::RWP * 2 + 16 <= (size_t)G::RAW_BYTES, "gauss second row smem");
        REQUIRE(2 * r + 1 < G::NR, "gauss staged row %d of %d", 2 * r + 1, G::NR);
      } else if (outside) {
        const size_t eoff = (size_t)(ra * G::RWP + (gx < 0 ? 0 : W - 1) - (x0 - G::RA)) * 2;
        REQUIRE(eoff + 2 <= (size_t)G::RAW_BYTES, "edge pixel smem");
        const int ecol = (gx < 0 ? 0 : W - 1) - (x0 - G::RA);
        REQUIRE(ecol >= 0 && ecol < G::SW, "edge column %d outside the staged row", ecol);
        const int ev = ecol / 8;  // the vector holding the edge pixel is copied, not filled
        const int egx = x0 - G::RA + 8 * ev;
        REQUIRE(egx >= 0 && egx < W, "edge pixel's vector not copied");
      }
      // the Gaussian's conversion of the landed tile
      if (OP == GAUSS) {
        const int yp = q % G::NP, cv = q / G::NP;
        const int cgx = x0 - G::RA + 8 * cv;
        int col = 8 * cv;
        if (cgx < 0 || cgx >= W) col = (cgx < 0 ? 0 : W - 1) - (x0 - G::RA);
        const size_t crd = (size_t)((2 * yp) * G::RWP + col) * 2, cwr = (size_t)(yp * G::CW + 8 * cv) * 8;
        REQUIRE(crd + G::RWP * 2 + 16 <= (size_t)G::RAW_BYTES, "convert read");
        REQUIRE(cwr + 64 <= (size_t)G::CV_BYTES, "convert write");
      }
    }
    // X task
    if (tid < G::XTASKS) {
      const int q = tid;
      if (OP == GAUSS) {
        const int xr = q % G::NP, xsg = q / G::NP;
        constexpr int E0 = G::XOFF & ~1;
        const size_t xrd = (size_t)(xr * G::CW + 8 * xsg + E0) * 8;
        const size_t xwr = (size_t)(xr * G::XP + 8 * xsg) * 4;
        REQUIRE(xrd + (size_t)(G::NWX - E0) * 8 <= (size_t)G::CV_BYTES, "gauss X read");
        REQUIRE(8 * xsg + G::NWX <= G::CW, "gauss X read past the row");
        REQUIRE(xwr + 32 + (size_t)G::XHALF * 4 <= (size_t)G::XS_BYTES, "gauss X write");
      } else {
        constexpr int NSG = TX / MX;
        const int xsg = q % NSG, xr = q / NSG;
        const size_t xrd = (size_t)((G::PAIRS ? 2 * xr : xr) * G::RWP + MX * xsg) * 2;
        const size_t xwr = (size_t)(xr * G::XP + MX * xsg) * 2;
        const size_t rows = G::PAIRS ? 2 : 1;
        REQUIRE(xrd + (rows - 1) * G::RWP * 2 + (size_t)G::NWX * 2 <= (size_t)G::RAW_BYTES, "X read");
        REQUIRE(MX * xsg + G::NWX <= G::SW, "op %d R %d X read past the staged row (%d > %d)", OP, R,
                MX * xsg + G::NWX, G::SW);
        REQUIRE((G::PAIRS ? 2 * xr + 1 : xr) < G::NR, "X row");
        REQUIRE(xwr + MX * 2 + (G::PAIRS ? (size_t)G::XHALF * 2 : 0) <= (size_t)G::XS_BYTES, "X write");
      }
    }
    // Y task
    const int c = tid & 31, g = tid >> 5;
    if (SEGY * g < TY) {
      const size_t yrd = G::PAIRS ? (size_t)((SEGY * g / 2) * G::XP + 2 * c) * G::XEL
                                  : (size_t)((SEGY * g) * G::XP + 2 * c) * G::XEL;
      for (int k = 0; k < SEGY + 2 * R; ++k) {
        const size_t off = G::PAIRS ? (size_t)((k & 1) * G::XHALF + (k >> 1) * G::XP) * G::XEL
                                    : (size_t)k * G::XP * G::XEL;
        const size_t w = OP == GAUSS ? 8 : 4;
        REQUIRE(yrd + off + w <= (size_t)G::XS_BYTES, "Y read row %d", SEGY * g + k);
        REQUIRE(SEGY * g + k < G::NR, "Y row %d of %d", SEGY * g + k, G::NR);
      }
    }
  }
  REQUIRE((size_t)G::SMEM <= 220 * 1024, "shared memory %d", G::SMEM);
  REQUIRE(RAWTOT + 2 * (size_t)G::CV_BYTES + 2 * (size_t)G::XS_BYTES == (size_t)G::SMEM, "buffer sum");
}

template <int OP, int R, int CZ> void check_shapes() {
  using C = typename DefaultCfg<OP, CZ>::type;
  const int ws[] = {8, 16, 64, 72, 128, 200, 1024};
  const int hs[] = {1, 2, 3, 31, 33, 70, 1024};
  for (int W : ws)
    for (int H : hs) {
      const int tx = (W + TX - 1) / TX, ty = (H + C::TY - 1) / C::TY;
      for (int by = 0; by < ty; by += (ty > 3 ? ty - 1 : 1))
        for (int bx = 0; bx < tx; bx += (tx > 3 ? tx - 1 : 1)) {
          check_cta<OP, R, CZ, C>(W, H, bx, by);
          if (g_fail) return;
        }
    }
}

template <int OP, int R, int CZ> void each_cz() {
  if constexpr (CZ >= 0) {
    check_shapes<OP, R, CZ>();
    each_cz<OP, R, CZ - 1>();
  }
}
template <int OP, int R, int CZMAX> void each_r() {
  if constexpr (R >= 1) {
    each_cz<OP, R, CZMAX>();
    each_r<OP, R - 1, CZMAX>();
  }
}

int main() {
  each_r<MIN, kMaxRInt, kMaxCzInt>();
  each_r<MAX, kMaxRInt, kMaxCzInt>();
  each_r<MEAN, kMaxRInt, kMaxCzInt>();
  each_r<GAUSS, kMaxRGauss, kMaxCzGauss>();
  if (g_fail) return 1;
  std::printf("ok %lld checks\n", g_checks);
  return 0;
}
