// Host-side check of the staged median kernels' shared-memory layouts
// (clk_median_impl.cuh: box27_staged_tile, sphere33_staged_tile,
// sphere33_staged_f32_tile).  For every CTA of a range of image extents it
// replays what the kernel's threads stage (cp.async vectors inside the row,
// edge-pixel fills outside it) into a model of each plane buffer, recording
// which clamped image pixel every shared-memory element holds, then replays
// every read of the tile body and checks that it stays inside the buffer and
// finds the pixel the reference's clamped read names: (clamp(y+dy),
// clamp(x+dx)) of plane clamp(z).  It also replays the z-pair loops' plane
// ring (which plane each buffer holds when it is read).  Built and run by
// tests/test_median_layout.py on the CPU; prints "ok" and exits 0, or reports
// the first bad access and exits 1.
#include <cstdio>
#include <vector>

#include "clk_median_impl.cuh"

using namespace clk::med;

static long long g_checks = 0;
static int g_fail = 0;

#define REQUIRE(cond, ...)                        \
  do {                                            \
    ++g_checks;                                   \
    if (!(cond)) {                                \
      if (!g_fail) {                              \
        std::printf("FAIL %s:%d: ", __FILE__, __LINE__); \
        std::printf(__VA_ARGS__);                 \
        std::printf("\n");                        \
      }                                           \
      g_fail = 1;                                 \
      return;                                     \
    }                                             \
  } while (0)

static int hclamp(int v, int hi) { return v < 0 ? 0 : v > hi ? hi : v; }

// a staged plane buffer: for each element the (row, column) of the image
// pixel it holds, or (-1, -1) if nothing was written
struct Plane {
  std::vector<int> row, col;
  Plane(int n) : row(n, -1), col(n, -1) {}
};

// Staging of one plane, as stage_plane_async + fill_plane (16-bit pixels,
// NR rows from y0 - HY, columns x0 - 8 .. x0 + SMW - 9) or the float kernel's
// stage (rows y0 - 2, columns x0 - 4 .. x0 + FSW - 5).  vec = pixels per
// 16-byte vector, width = pixels per staged row, margin = staged columns left
// of x0.
static void stage(Plane& p, int nr, int hy, int vec, int width, int margin, int x0, int y0, int W, int H) {
  const int nv = width / vec;
  for (int t = 0; t < BX * BY; ++t) {
    if (t >= nr * nv) continue;
    const int r = t / nv, v = t - r * nv;
    const int gx = x0 - margin + vec * v;
    const int gy = hclamp(y0 - hy + r, H - 1);
    for (int e = 0; e < vec; ++e) {
      const size_t off = (size_t)r * width + vec * v + e;
      if (off >= p.row.size()) { g_fail = 1; std::printf("FAIL staging offset %zu of %zu\n", off, p.row.size()); return; }
      if (gx >= 0 && gx < W) {
        if (gx + vec > W) { g_fail = 1; std::printf("FAIL vector past the row end (gx %d W %d)\n", gx, W); return; }
        p.row[off] = gy, p.col[off] = gx + e;
      } else {
        p.row[off] = gy, p.col[off] = gx < 0 ? 0 : W - 1;  // the row's edge pixel
      }
    }
  }
}

// a read of element `off` of plane buffer p must hold image pixel (gy, gx)
#define READ(p, off, gy, gx, what)                                                                       \
  do {                                                                                                  \
    const size_t o_ = (size_t)(off);                                                                    \
    REQUIRE(o_ < (p).row.size(), "%s: offset %zu of %zu", what, o_, (p).row.size());                    \
    REQUIRE((p).row[o_] == (gy) && (p).col[o_] == (gx), "%s: holds (%d, %d), wants (%d, %d)", what,     \
            (p).row[o_], (p).col[o_], (gy), (gx));                                                      \
  } while (0)

// box27_staged_tile: rows y0-1 .. y0+BYP, 64 + 16 columns; thread (px, py)
// reads rows y-1 .. y+2 (y = y0 + 2 py), pixel words (x-2, x-1), (x, x+1),
// (x+2, x+3)
static void check_box(int W, int H, int bx, int by) {
  const int x0 = bx * 2 * BX, y0 = by * BYP;
  Plane p(SMR * SMW);
  stage(p, SMR, 1, 8, SMW, 8, x0, y0, W, H);
  if (g_fail) return;
  for (int t = 0; t < BX * BY; ++t) {
    const int px = t % BX, py = t / BX, x = x0 + 2 * px, y = y0 + 2 * py;
    for (int r = 0; r < 4; ++r)
      for (int wv = 0; wv < 3; ++wv)
        for (int e = 0; e < 2; ++e) {
          const int off = (2 * py + r) * SMW + 2 * (px + 3 + wv) + e;
          READ(p, off, hclamp(y - 1 + r, H - 1), hclamp(x - 2 + 2 * wv + e, W - 1), "box row word");
        }
  }
}

// sphere33_staged_tile: rows y0-2 .. y0+BY+1; thread reads rows y-2 .. y+2,
// pixel words (x-2, x-1), (x, x+1), (x+2, x+3)
static void check_sphere16(int W, int H, int bx, int by) {
  const int x0 = bx * 2 * BX, y0 = by * BY;
  Plane p(SPR * SMW);
  stage(p, SPR, 2, 8, SMW, 8, x0, y0, W, H);
  if (g_fail) return;
  for (int t = 0; t < BX * BY; ++t) {
    const int px = t % BX, py = t / BX, x = x0 + 2 * px, y = y0 + py;
    for (int dy = -2; dy <= 2; ++dy)
      for (int wv = 0; wv < 3; ++wv)
        for (int e = 0; e < 2; ++e) {
          const int off = (py + 2 + dy) * SMW + 2 * (px + 3 + wv) + e;
          READ(p, off, hclamp(y + dy, H - 1), hclamp(x - 2 + 2 * wv + e, W - 1), "sphere row word");
        }
  }
}

// sphere33_staged_f32_tile: rows y0-2 .. y0+BY+1, columns x0-4 .. x0+35;
// thread reads columns x-2 .. x+2 of rows y-2 .. y+2
static void check_sphere32(int W, int H, int bx, int by) {
  const int x0 = bx * BX, y0 = by * BY;
  Plane p(SPR * FSW);
  stage(p, SPR, 2, 4, FSW, 4, x0, y0, W, H);
  if (g_fail) return;
  for (int t = 0; t < BX * BY; ++t) {
    const int px = t % BX, py = t / BX, x = x0 + px, y = y0 + py;
    for (int dy = -2; dy <= 2; ++dy)
      for (int dx = -2; dx <= 2; ++dx) {
        const int off = (py + 2 + dy) * FSW + px + 4 + dx;
        READ(p, off, hclamp(y + dy, H - 1), hclamp(x + dx, W - 1), "float sphere key");
      }
  }
}

// The plane rings of the z-pair loops: which image plane each buffer holds
// when a pair reads it.  Box: buffers 0, 1 hold z0-1, z0; the pair zo reads
// buffers slot, slot+1 (planes zo+1, zo+2) and stages zo+3, zo+4 into the
// other two.  Sphere: buffer (z - z0 + 2) & 7 holds plane z; the pair zo
// reads planes zo-1 .. zo+4 and stages zo+5, zo+6.
static void check_rings(int D, int zchunk) {
  for (int z0 = 0; z0 < D; z0 += zchunk) {
    const int z1 = z0 + zchunk < D ? z0 + zchunk : D;
    {  // box
      int held[4];
      held[0] = z0 - 1, held[1] = z0, held[2] = z0 + 1, held[3] = z0 + 2;
      int slot = 2;
      for (int zo = z0; zo < z1; zo += 2) {
        REQUIRE(held[slot] == zo + 1 && held[slot + 1] == zo + 2, "box ring at zo %d", zo);
        const int nslot = slot ^ 2;
        if (zo + 2 < z1) held[nslot] = zo + 3, held[nslot + 1] = zo + 4;
        slot = nslot;
      }
    }
    {  // sphere (both pixel types)
      int held[8];
      for (int k = 0; k < 8; ++k) held[k] = -1000;
      auto slot = [&](int z) { return (z - z0 + 2) & 7; };
      for (int z = z0 - 2; z <= z0 + 4; ++z) held[slot(z)] = z;
      for (int zo = z0; zo < z1; zo += 2) {
        for (int z = zo - 1; z <= zo + 4; ++z) REQUIRE(held[slot(z)] == z, "sphere ring: plane %d at zo %d", z, zo);
        // the prologue and the previous pair read zo-3, zo-2 last: their
        // buffers take zo+5, zo+6
        if (zo + 2 < z1) {
          REQUIRE(slot(zo + 5) == slot(zo - 3) && slot(zo + 6) == slot(zo - 2), "sphere ring reuse at zo %d", zo);
          held[slot(zo + 5)] = zo + 5, held[slot(zo + 6)] = zo + 6;
        }
      }
    }
  }
}

int main() {
  const int ws16[] = {8, 16, 64, 72, 128, 136, 200};
  const int ws32[] = {4, 8, 12, 32, 36, 100, 132};
  const int hs[] = {1, 2, 3, 7, 8, 9, 16, 17, 33, 70};
  for (int W : ws16)
    for (int H : hs) {
      const int tx = (W + 2 * BX - 1) / (2 * BX);
      for (int bx = 0; bx < tx && !g_fail; ++bx) {
        for (int by = 0; by < (H + BYP - 1) / BYP && !g_fail; ++by) check_box(W, H, bx, by);
        for (int by = 0; by < (H + BY - 1) / BY && !g_fail; ++by) check_sphere16(W, H, bx, by);
      }
    }
  for (int W : ws32)
    for (int H : hs)
      for (int bx = 0; bx < (W + BX - 1) / BX && !g_fail; ++bx)
        for (int by = 0; by < (H + BY - 1) / BY && !g_fail; ++by) check_sphere32(W, H, bx, by);
  for (int D : {1, 2, 3, 5, 16, 33, 256})
    for (int zc : {2, 4, 6, 16, 64, 256})
      if (!g_fail) check_rings(D, zc);
  if (g_fail) return 1;
  std::printf("ok %lld checks\n", g_checks);
  return 0;
}
