// dml_config.cpp - initial configurations (host code).
//
// pos_inic (src/dana.F90:330-396) places ions by random sequential addition
// with an O(N^2) overlap scan and cannot load an electrode.  These
// generators build the frozen bcc Li slab and RSA ions with a cell grid
// (O(N)), drawing from the keyed Philox stream so a configuration is a pure
// function of its seed.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "../../include/dml.h"
#include "../../include/dml_rng.h"

extern "C" {

int dml_gen_bcc_slab(int32_t nx, int32_t ny, int32_t nz, double a, double* pos_out, int32_t cap) {
  int64_t n = 2LL * nx * ny * nz;
  if (nx <= 0 || ny <= 0 || nz <= 0 || a <= 0) return -DML_E_ARG;
  if (n > cap) return -DML_E_CAPACITY;
  int64_t q = 0;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        pos_out[3 * q + 0] = i * a;
        pos_out[3 * q + 1] = j * a;
        pos_out[3 * q + 2] = k * a;
        ++q;
        pos_out[3 * q + 0] = (i + 0.5) * a;
        pos_out[3 * q + 1] = (j + 0.5) * a;
        pos_out[3 * q + 2] = (k + 0.5) * a;
        ++q;
      }
  return (int)n;
}

// n ions uniform in [0,box_x) x [0,box_y) x [zlo,zhi) with pairwise minimum
// image distance >= dmin in x,y (z not periodic).  Returns 0 or -status.
int dml_gen_ions(uint64_t seed, int32_t n, double box_x, double box_y, double zlo, double zhi,
                 double dmin, double* pos_out) {
  if (n < 0 || !(box_x > 0) || !(box_y > 0) || !(zhi > zlo) || dmin < 0) return -DML_E_ARG;
  double cs = dmin > 0 ? dmin : 1.0;
  int gx = std::max(1, (int)(box_x / cs)), gy = std::max(1, (int)(box_y / cs));
  int gz = std::max(1, (int)((zhi - zlo) / cs));
  double cx = box_x / gx, cy = box_y / gy, cz = (zhi - zlo) / gz;
  std::vector<std::vector<int>> grid((size_t)gx * gy * gz);
  const double d2 = dmin * dmin;
  for (int i = 0; i < n; ++i) {
    bool placed = false;
    for (int t = 0; t < 10000 && !placed; ++t) {
      dml_u4 w = dml_draw(seed, (int64_t)t, (uint64_t)i, DML_RNG_INIT, 0);
      dml_u4 w2 = dml_draw(seed, (int64_t)t, (uint64_t)i, DML_RNG_INIT, 1);
      double x = dml_u53(w.w[0], w.w[1]) * box_x;
      double y = dml_u53(w.w[2], w.w[3]) * box_y;
      double z = zlo + dml_u53(w2.w[0], w2.w[1]) * (zhi - zlo);
      int ix = std::min(gx - 1, (int)(x / cx)), iy = std::min(gy - 1, (int)(y / cy));
      int iz = std::min(gz - 1, (int)((z - zlo) / cz));
      // distinct neighbour cells (fewer than 3 cells: every cell once)
      int xs[3], ys[3], nxs = 0, nys = 0;
      if (gx >= 3) {
        for (int dx = -1; dx <= 1; ++dx) xs[nxs++] = ((ix + dx) % gx + gx) % gx;
      } else {
        for (int xx = 0; xx < gx; ++xx) xs[nxs++] = xx;
      }
      if (gy >= 3) {
        for (int dy = -1; dy <= 1; ++dy) ys[nys++] = ((iy + dy) % gy + gy) % gy;
      } else {
        for (int yy = 0; yy < gy; ++yy) ys[nys++] = yy;
      }
      bool ok = true;
      for (int dz = -1; dz <= 1 && ok; ++dz) {
        int zz = iz + dz;
        if (zz < 0 || zz >= gz) continue;
        for (int a = 0; a < nys && ok; ++a)
          for (int b = 0; b < nxs && ok; ++b)
            for (int q : grid[((size_t)zz * gy + ys[a]) * gx + xs[b]]) {
              double vx = x - pos_out[3 * q], vy = y - pos_out[3 * q + 1], vz = z - pos_out[3 * q + 2];
              vx -= box_x * std::round(vx / box_x);
              vy -= box_y * std::round(vy / box_y);
              if (vx * vx + vy * vy + vz * vz < d2) {
                ok = false;
                break;
              }
            }
      }
      if (ok) {
        pos_out[3 * i] = x;
        pos_out[3 * i + 1] = y;
        pos_out[3 * i + 2] = z;
        grid[((size_t)iz * gy + iy) * gx + ix].push_back(i);
        placed = true;
      }
    }
    if (!placed) return -DML_E_RSA;
  }
  return 0;
}

}  // extern "C"
