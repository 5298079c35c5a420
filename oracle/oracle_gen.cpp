// oracle_gen.cpp - TEST INFRASTRUCTURE ONLY: serial generators of initial
// configurations, the checker of the device generator (dml_gen_ions) and
// the source of the inputs that tests and the CPU baseline feed to both
// sides.  Never linked into the product.
//
// Random sequential addition as pos_inic does it (src/dana.F90:361-389):
// ion i tries points one after another and keeps the first whose minimum-
// image distance to every ion placed before it is at least dmin, giving up
// after 10 000 tries ("demasiados intentos", :386-389).  Two changes from
// the reference, shared with the device: the k-th try of ion i is the keyed
// Philox draw (seed, step k, id i, DML_RNG_INIT) instead of ran(), and the
// earlier ions are looked up in a cell grid (cell edge >= dmin, the 27 cells
// around the try; every cell once along an axis of fewer than 3 cells)
// instead of the reference's O(N^2) scan.  The distance is
//   vd = p - q;  vd(l) -= box(l) * round(vd(l) / box(l)) for x, y;
//   d2 = (vd_x^2 + vd_y^2) + vd_z^2,  rejected when d2 < dmin^2,
// evaluated without contraction (-ffp-contract=off).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "../include/dml.h"
#include "../include/dml_rng.h"

extern "C" {

// The 2*nx*ny*nz atoms of a bcc lattice of constant a: per cell the corner,
// then the body centre; x fastest, then y, then z.  Returns the count or
// -status.
int orc_gen_bcc_slab(int32_t nx, int32_t ny, int32_t nz, double a, double* pos_out,
                     int32_t cap) {
  if (nx <= 0 || ny <= 0 || nz <= 0 || !(a > 0)) return -DML_E_ARG;
  const int64_t total = 2LL * nx * ny * nz;
  if (total > cap) return -DML_E_CAPACITY;
  double* p = pos_out;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        p[0] = i * a;
        p[1] = j * a;
        p[2] = k * a;
        p[3] = (i + 0.5) * a;
        p[4] = (j + 0.5) * a;
        p[5] = (k + 0.5) * a;
        p += 6;
      }
  return (int)total;
}

// n ions in [0,box_x) x [0,box_y) x [zlo,zhi), pairwise minimum-image
// distance >= dmin (x, y periodic, z not).  Returns 0 or -status
// (-DML_E_RSA when an ion finds no place in 10 000 tries).
int orc_gen_ions(uint64_t seed, int32_t n, double box_x, double box_y, double zlo, double zhi,
                 double dmin, double* pos_out) {
  if (n < 0 || !(box_x > 0) || !(box_y > 0) || !(zhi > zlo) || dmin < 0) return -DML_E_ARG;
  const double edge = dmin > 0 ? dmin : 1.0;
  const int gx = std::max(1, (int)(box_x / edge));
  const int gy = std::max(1, (int)(box_y / edge));
  const int gz = std::max(1, (int)((zhi - zlo) / edge));
  const double cx = box_x / gx, cy = box_y / gy, cz = (zhi - zlo) / gz;
  const double d2 = dmin * dmin;
  // cell chains: head per cell, next per ion
  std::vector<int> head((size_t)gx * gy * gz, -1), next((size_t)n, -1);
  auto axis_cells = [](int c, int g, int* out) {
    int k = 0;
    if (g >= 3) {
      for (int d = -1; d <= 1; ++d) out[k++] = ((c + d) % g + g) % g;
    } else {
      for (int q = 0; q < g; ++q) out[k++] = q;
    }
    return k;
  };
  for (int i = 0; i < n; ++i) {
    int t = 0;
    for (; t < 10000; ++t) {
      dml_u4 a = dml_draw(seed, (int64_t)t, (uint64_t)i, DML_RNG_INIT, 0);
      dml_u4 b = dml_draw(seed, (int64_t)t, (uint64_t)i, DML_RNG_INIT, 1);
      const double x = dml_u53(a.w[0], a.w[1]) * box_x;
      const double y = dml_u53(a.w[2], a.w[3]) * box_y;
      const double z = zlo + dml_u53(b.w[0], b.w[1]) * (zhi - zlo);
      const int ix = std::min(gx - 1, (int)(x / cx));
      const int iy = std::min(gy - 1, (int)(y / cy));
      const int iz = std::min(gz - 1, (int)((z - zlo) / cz));
      int xs[3], ys[3];
      const int nxs = axis_cells(ix, gx, xs), nys = axis_cells(iy, gy, ys);
      bool clash = false;
      for (int dz = -1; dz <= 1 && !clash; ++dz) {
        const int zz = iz + dz;
        if (zz < 0 || zz >= gz) continue;
        for (int u = 0; u < nys && !clash; ++u)
          for (int v = 0; v < nxs && !clash; ++v)
            for (int q = head[((size_t)zz * gy + ys[u]) * gx + xs[v]]; q >= 0; q = next[q]) {
              double vx = x - pos_out[3 * q];
              double vy = y - pos_out[3 * q + 1];
              const double vz = z - pos_out[3 * q + 2];
              vx -= box_x * std::round(vx / box_x);
              vy -= box_y * std::round(vy / box_y);
              if (vx * vx + vy * vy + vz * vz < d2) {
                clash = true;
                break;
              }
            }
      }
      if (!clash) {
        pos_out[3 * i] = x;
        pos_out[3 * i + 1] = y;
        pos_out[3 * i + 2] = z;
        const size_t c = ((size_t)iz * gy + iy) * gx + ix;
        next[i] = head[c];
        head[c] = i;
        break;
      }
    }
    if (t == 10000) return -DML_E_RSA;
  }
  return 0;
}

}  // extern "C"
