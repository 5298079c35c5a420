// dml_gen.cu - initial configurations: the frozen bcc electrode (host) and
// random sequential addition of ions on the GPU.
//
// pos_inic (src/dana.F90:330-396) places ions by random sequential addition:
// ion i keeps the first try whose minimum-image distance to every ion placed
// before it is at least the separation (:361-389), with an O(N^2) scan per
// try.  The device generator gives exactly that sequential result for many
// systems at once, one thread block per system:
//
//  - the k-th try of ion i is the keyed Philox draw (seed, k, i,
//    DML_RNG_INIT), so any thread can form any ion's tries;
//  - placed ions sit in chains over a cell grid of edge >= the separation,
//    and a try is tested against the chains of its 27 cells (every cell once
//    along an axis of fewer than 3 cells);
//  - a round takes the window of the next 256 unplaced ions.  Each thread
//    advances its ion to the first try that clears every placed ion (all of
//    them earlier in the order).  Then each try is tested against the tries
//    of the earlier ions of the window.  Ions before the first one whose try
//    meets an earlier window try are placed (nothing earlier can reject
//    them), and that first one's try is rejected (the ion it meets is now
//    placed).  Every round places at least the window's first ion.
//
// Results are bit-identical to the serial rule: the distance is evaluated
// with the same operations in the same order (no contraction, compiled with
// --fmad=false), and the grid is the same.  An FP32 screen on z (with a
// margin that bounds its rounding) skips the FP64 test for window pairs that
// are far apart along z.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "../../include/dml.h"
#include "../../include/dml_rng.h"

namespace {

constexpr int kGenW = 256;        // ions per round and block
constexpr int kGenTries = 10000;  // tries per ion (src/dana.F90:365)
constexpr long long kGenMaxCells = 1LL << 28;

struct GenSys {
  unsigned long long seed;
  int n, gx, gy, gz;
  double bx, by, zlo, zhi, d2, cx, cy, cz;
  float sepf;          // FP32 z gap beyond which two points are surely apart
  long long off;       // first ion of this system (output, chains, tries)
  long long cell_off;  // first cell of this system
};

__device__ __forceinline__ void gen_try(const GenSys& S, int i, int t, double& x, double& y,
                                        double& z) {
  dml_u4 a = dml_draw(S.seed, (int64_t)t, (uint64_t)i, DML_RNG_INIT, 0);
  dml_u4 b = dml_draw(S.seed, (int64_t)t, (uint64_t)i, DML_RNG_INIT, 1);
  x = dml_u53(a.w[0], a.w[1]) * S.bx;
  y = dml_u53(a.w[2], a.w[3]) * S.by;
  z = S.zlo + dml_u53(b.w[0], b.w[1]) * (S.zhi - S.zlo);
}

// Minimum image in x and y, squared distance below the separation.
__device__ __forceinline__ bool gen_clash(const GenSys& S, double x, double y, double z, double qx,
                                          double qy, double qz) {
  double vx = x - qx;
  double vy = y - qy;
  const double vz = z - qz;
  vx -= S.bx * round(vx / S.bx);
  vy -= S.by * round(vy / S.by);
  return vx * vx + vy * vy + vz * vz < S.d2;
}

__device__ __forceinline__ int gen_axis(int c, int g, int* out) {
  if (g >= 3) {
    out[0] = c == 0 ? g - 1 : c - 1;
    out[1] = c;
    out[2] = c == g - 1 ? 0 : c + 1;
    return 3;
  }
  for (int q = 0; q < g; ++q) out[q] = q;
  return g;
}

__device__ __forceinline__ long long gen_cell(const GenSys& S, double x, double y, double z,
                                              int& ix, int& iy, int& iz) {
  ix = min(S.gx - 1, (int)(x / S.cx));
  iy = min(S.gy - 1, (int)(y / S.cy));
  iz = min(S.gz - 1, (int)((z - S.zlo) / S.cz));
  return ((long long)iz * S.gy + iy) * S.gx + ix;
}

// Does (x, y, z) lie within the separation of a placed ion?  Chains are
// acyclic (each ion enters one chain once); the walk is bounded anyway.
__device__ bool gen_grid_clash(const GenSys& S, const int* head, const int* next,
                               const double* out, double x, double y, double z) {
  int ix, iy, iz;
  gen_cell(S, x, y, z, ix, iy, iz);
  int xs[3], ys[3];
  const int nxs = gen_axis(ix, S.gx, xs), nys = gen_axis(iy, S.gy, ys);
  for (int dz = -1; dz <= 1; ++dz) {
    const int zz = iz + dz;
    if (zz < 0 || zz >= S.gz) continue;
    for (int u = 0; u < nys; ++u)
      for (int v = 0; v < nxs; ++v) {
        int q = head[((long long)zz * S.gy + ys[u]) * S.gx + xs[v]];
        for (int walk = 0; q >= 0 && walk < S.n; ++walk) {
          if (gen_clash(S, x, y, z, out[3 * (long long)q], out[3 * (long long)q + 1],
                        out[3 * (long long)q + 2]))
            return true;
          q = next[q];
        }
      }
  }
  return false;
}

__global__ void __launch_bounds__(kGenW) rsa_kernel(const GenSys* sys, double* out, int* head,
                                                    int* next, int* tries, int* status) {
  const GenSys S = sys[blockIdx.x];
  __shared__ double sx[kGenW], sy[kGenW], sz[kGenW];
  __shared__ float szf[kGenW];
  __shared__ int s_first, s_fail;
  double* o = out + 3 * S.off;
  int* hd = head + S.cell_off;
  int* nx = next + S.off;
  int* tr = tries + S.off;
  const int tid = threadIdx.x;
  int placed = 0;
  // every round places at least one ion, so n rounds suffice
  for (int round = 0; round < S.n && placed < S.n; ++round) {
    const int i = placed + tid;
    const bool have = i < S.n;
    if (tid == 0) {
      s_first = kGenW;
      s_fail = 0;
    }
    int t = 0;
    double x = 0.0, y = 0.0, z = 0.0;
    bool ok = false;
    if (have) {
      for (t = tr[i]; t < kGenTries; ++t) {
        gen_try(S, i, t, x, y, z);
        if (!gen_grid_clash(S, hd, nx, o, x, y, z)) {
          ok = true;
          break;
        }
      }
      sx[tid] = x;
      sy[tid] = y;
      sz[tid] = z;
      szf[tid] = (float)z;
    }
    __syncthreads();
    // An ion whose every try meets an earlier placed ion fails the serial
    // rule too (there it meets the same ions and more).
    if (have && !ok) atomicOr(&s_fail, 1);
    if (have && ok) {
      const float zf = szf[tid];
      for (int j = 0; j < tid; ++j) {
        if (fabsf(zf - szf[j]) >= S.sepf) continue;
        if (gen_clash(S, x, y, z, sx[j], sy[j], sz[j])) {
          atomicMin(&s_first, tid);
          break;
        }
      }
    }
    __syncthreads();
    if (s_fail) {
      if (tid == 0) status[blockIdx.x] = DML_E_RSA;
      return;
    }
    const int first = s_first;
    if (have) {
      if (tid < first) {
        o[3 * (long long)i] = x;
        o[3 * (long long)i + 1] = y;
        o[3 * (long long)i + 2] = z;
        int ix, iy, iz;
        const long long c = gen_cell(S, x, y, z, ix, iy, iz);
        nx[i] = atomicExch(&hd[c], i);
      } else {
        tr[i] = tid == first ? t + 1 : t;
      }
    }
    __syncthreads();
    placed += min(first, S.n - placed);
  }
  if (tid == 0) status[blockIdx.x] = placed == S.n ? 0 : DML_E_RSA;
}

template <class T>
int gen_alloc(T** p, size_t n, std::vector<void*>& keep) {
  if (n == 0) n = 1;
  if (cudaMalloc((void**)p, n * sizeof(T)) != cudaSuccess) return DML_E_NOMEM;
  keep.push_back(*p);
  return 0;
}

}  // namespace

extern "C" {

int dml_gen_bcc_slab(int32_t nx, int32_t ny, int32_t nz, double a, double* pos_out, int32_t cap) {
  if (nx <= 0 || ny <= 0 || nz <= 0 || !(a > 0)) return -DML_E_ARG;
  const int64_t total = 2LL * nx * ny * nz;
  if (total > cap) return -DML_E_CAPACITY;
  int64_t q = 0;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const double c[6] = {i * a, j * a, k * a, (i + 0.5) * a, (j + 0.5) * a, (k + 0.5) * a};
        for (int m = 0; m < 6; ++m) pos_out[6 * q + m] = c[m];
        ++q;
      }
  return (int)total;
}

int dml_gen_ions_batch(int32_t n_sys, const dml_ion_spec* specs, double* pos_out,
                       int32_t* status) {
  if (n_sys < 0 || (n_sys > 0 && (!specs || !pos_out))) return DML_E_ARG;
  std::vector<GenSys> sys((size_t)n_sys);
  long long n_tot = 0, cells = 0;
  for (int s = 0; s < n_sys; ++s) {
    const dml_ion_spec& q = specs[s];
    if (q.n < 0 || !(q.box_x > 0) || !(q.box_y > 0) || !(q.zhi > q.zlo) || !(q.dmin >= 0))
      return DML_E_ARG;
    GenSys& S = sys[s];
    const double edge = q.dmin > 0 ? q.dmin : 1.0;
    S.seed = q.seed;
    S.n = q.n;
    // cells of the serial rule: int(extent / edge) per axis, at least one
    const double ex = q.box_x / edge, ey = q.box_y / edge, ez = (q.zhi - q.zlo) / edge;
    if (!(ex < 1e9 && ey < 1e9 && ez < 1e9)) return DML_E_CAPACITY;
    S.gx = std::max(1, (int)ex);
    S.gy = std::max(1, (int)ey);
    S.gz = std::max(1, (int)ez);
    S.bx = q.box_x;
    S.by = q.box_y;
    S.zlo = q.zlo;
    S.zhi = q.zhi;
    S.d2 = q.dmin * q.dmin;
    S.cx = q.box_x / S.gx;
    S.cy = q.box_y / S.gy;
    S.cz = (q.zhi - q.zlo) / S.gz;
    // z rounded to FP32 is within 2^-24 |z| of z; the float difference of
    // two such values is within 3 * 2^-24 * max|z| of the true gap
    const double zabs = std::max(std::fabs(q.zlo), std::fabs(q.zhi));
    S.sepf = std::nextafter((float)(q.dmin + 4e-7 * zabs + 1e-6), INFINITY);
    S.off = n_tot;
    S.cell_off = cells;
    n_tot += q.n;
    cells += (long long)S.gx * S.gy * S.gz;
    if (cells > kGenMaxCells || n_tot > INT32_MAX) return DML_E_CAPACITY;
  }
  if (n_tot == 0) {  // nothing to place: no device work
    if (status)
      for (int s = 0; s < n_sys; ++s) status[s] = 0;
    return 0;
  }
  std::vector<void*> keep;
  GenSys* d_sys = nullptr;
  double* d_out = nullptr;
  int *d_head = nullptr, *d_next = nullptr, *d_tries = nullptr, *d_status = nullptr;
  int rc = 0;
  if ((rc = gen_alloc(&d_sys, n_sys, keep)) || (rc = gen_alloc(&d_out, 3 * n_tot, keep)) ||
      (rc = gen_alloc(&d_head, cells, keep)) || (rc = gen_alloc(&d_next, n_tot, keep)) ||
      (rc = gen_alloc(&d_tries, n_tot, keep)) || (rc = gen_alloc(&d_status, n_sys, keep))) {
    for (void* p : keep) cudaFree(p);
    return rc;
  }
  std::vector<int> st((size_t)n_sys, 0);
  bool ok = cudaMemcpy(d_sys, sys.data(), sizeof(GenSys) * n_sys, cudaMemcpyHostToDevice) ==
                cudaSuccess &&
            cudaMemset(d_head, 0xff, sizeof(int) * std::max(1LL, cells)) == cudaSuccess &&
            cudaMemset(d_tries, 0, sizeof(int) * std::max(1LL, n_tot)) == cudaSuccess &&
            cudaMemset(d_status, 0, sizeof(int) * n_sys) == cudaSuccess;
  if (ok) {
    rsa_kernel<<<n_sys, kGenW>>>(d_sys, d_out, d_head, d_next, d_tries, d_status);
    ok = cudaGetLastError() == cudaSuccess &&
         cudaMemcpy(st.data(), d_status, sizeof(int) * n_sys, cudaMemcpyDeviceToHost) ==
             cudaSuccess &&
         cudaMemcpy(pos_out, d_out, sizeof(double) * 3 * n_tot, cudaMemcpyDeviceToHost) ==
             cudaSuccess;
  }
  for (void* p : keep) cudaFree(p);
  if (!ok) return DML_E_CUDA;
  rc = 0;
  for (int s = 0; s < n_sys; ++s) {
    if (status) status[s] = st[s];
    if (!rc && st[s]) rc = st[s];
  }
  return rc;
}

int dml_gen_ions(uint64_t seed, int32_t n, double box_x, double box_y, double zlo, double zhi,
                 double dmin, double* pos_out) {
  dml_ion_spec q;
  q.seed = seed;
  q.n = n;
  q.pad = 0;
  q.box_x = box_x;
  q.box_y = box_y;
  q.zlo = zlo;
  q.zhi = zhi;
  q.dmin = dmin;
  const int rc = dml_gen_ions_batch(1, &q, pos_out, nullptr);
  return rc ? -rc : 0;
}

}  // extern "C"
