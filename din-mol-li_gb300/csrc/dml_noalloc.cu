// dml_noalloc.cu - dml_force_noalloc: the plain FP64 pair force and energy
// (fuerza, src/dana.F90:1055-1139) over caller-provided arrays, for callers
// that cannot allocate device memory.
//
// Who cannot allocate: a host program whose device memory belongs to another
// allocator or runtime (a Fortran driver whose arrays a CUDA Fortran or
// OpenACC runtime owns, a framework whose caching allocator has reserved the
// free memory, so that a cudaMalloc of ours would fail); and a time-stepping
// loop that must not call cudaMalloc or cudaFree, because cudaFree waits for
// the whole device and both stall the host inside the loop.  Such a caller
// passes inputs and outputs it already owns; the scratch the kernels need --
// the per-atom buckets that order the interacting list entries, as in the
// context path -- lives in one file-scope static device array of fixed size.
//
// Limits: at most kNoallocMaxAtoms (16384) atoms and kNoallocEvCap (32)
// interacting list entries per atom per call; more atoms return
// DML_E_CAPACITY before anything is launched, more entries return
// DML_E_EVENT_OVERFLOW.  The array (about 25 MB) is held by every GPU that
// loads the library until the process exits.
//
// Set-up: the first call on a device (with that device current) takes the
// array's device address with cudaGetSymbolAddress and keeps it for later
// calls on that device; make that first call before any stream capture.  The
// kept address does not survive cudaDeviceReset (the module is loaded again
// afterwards at another address): do not call this after a reset.  All calls
// share the array and the array keeps the last call's contents: each call
// clears what must start at zero, and calls that overlap on the GPU
// (different streams, or host threads) race on it.  Each call ends by
// reading its status back to the host and waiting for its stream.  When the
// status is not 0, force and epot are left as the caller passed them.
// Compiled with --fmad=false, so results are bit-identical to dml_force on
// the same positions and lists.
#include <cuda_runtime.h>

#include <climits>
#include <mutex>

#include "../../include/dml.h"
#include "dml_internal.h"

namespace {

constexpr int kNoallocMaxAtoms = 16384;
constexpr int kNoallocEvCap = 32;

struct NoallocScratch {
  int error;
  int err_info;
  int pad[62];  // keeps the arrays below 256-byte aligned
  int ev_count[kNoallocMaxAtoms];
  int8_t is_ref[kNoallocMaxAtoms];
  dml::EvRec ev[(size_t)kNoallocMaxAtoms * kNoallocEvCap];
};

static __device__ __align__(256) NoallocScratch g_noalloc_scratch;

std::mutex g_addr_mu;
NoallocScratch* g_addr[64] = {nullptr};

__device__ __forceinline__ double dot3n(double x, double y, double z) { return (x * x + y * y) + z * z; }

__device__ __forceinline__ double pow6n(double x) {
  double x2 = x * x;
  double x4 = x2 * x2;
  return x2 * x4;
}
__device__ __forceinline__ double pow7n(double x) {
  double x2 = x * x;
  double x3 = x * x2;
  double x4 = x2 * x2;
  return x3 * x4;
}

struct NoallocParams {
  double box[2], halfbox[2];
  double eps[3][3], r0sq[3][3], b0[3][3], c0[3][3];
};

__global__ void noalloc_clear_kernel(NoallocScratch* sc, int n) {
  DML_GRID_WAIT();
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) {
    sc->error = 0;
    sc->err_info = 0;
  }
  if (i < n) {
    sc->ev_count[i] = 0;
    sc->is_ref[i] = 0;
  }
}

// One warp per hs%ref member; every interacting entry recorded for both
// atoms with the key (rank, jj) of the reference's accumulation order.
__device__ __forceinline__ void noalloc_fail(NoallocScratch* sc, int code, int info) {
  if (atomicCAS(&sc->error, 0, code) == 0) sc->err_info = info;
}

__global__ void noalloc_pairs_kernel(NoallocScratch* sc, NoallocParams p, int n_atoms, int n_ref,
                                     const double* pos, const int32_t* z, const int32_t* ref,
                                     const int32_t* nn, const int32_t* list, int ld) {
  DML_GRID_WAIT();
  int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (r >= n_ref) return;
  int h = ref[r];
  if (h < 0 || h >= n_atoms) return;  // reported by noalloc_ref_mark_kernel
  int k = z[h];
  if (k < 1 || k > 3) {
    if (lane == 0) noalloc_fail(sc, DML_E_ARG, h);
    return;
  }
  double xi = pos[3 * h], yi = pos[3 * h + 1], zi = pos[3 * h + 2];
  int n = nn[r];
  if (n < 0 || n > ld) {
    if (lane == 0) noalloc_fail(sc, DML_E_ARG, r);
    return;
  }
  for (int jj = lane; jj < n; jj += 32) {
    int j = list[(size_t)r * ld + jj];
    if (j < 0) continue;  // limbo
    if (j >= n_atoms) {
      noalloc_fail(sc, DML_E_ARG, r);
      continue;
    }
    int m = z[j];
    if (m < 1 || m > 3) {
      noalloc_fail(sc, DML_E_ARG, j);
      continue;
    }
    if (k == DML_Z_CG && m == DML_Z_CG) continue;
    double eps = p.eps[k - 1][m - 1];
    if (eps == 0.0) continue;  // signed zeros only
    double vx = xi - pos[3 * j], vy = yi - pos[3 * j + 1], vz = zi - pos[3 * j + 2];
    if (vx > p.halfbox[0]) {
      vx = vx - p.box[0];
    } else if (vx < -p.halfbox[0]) {
      vx = vx + p.box[0];
    }
    if (vy > p.halfbox[1]) {
      vy = vy - p.box[1];
    } else if (vy < -p.halfbox[1]) {
      vy = vy + p.box[1];
    }
    double dr = dot3n(vx, vy, vz);
    if (dr > p.r0sq[k - 1][m - 1]) continue;
    dr = sqrt(dr);
    double c = p.c0[k - 1][m - 1] / pow7n(dr);
    double b = p.b0[k - 1][m - 1] / pow6n(dr);
    double aux = c * (b - 1.0);
    dml::EvRec e;
    e.key = ((unsigned long long)(unsigned)r << 32) | (unsigned)jj;
    e.fx = aux * vx / dr;
    e.fy = aux * vy / dr;
    e.fz = aux * vz / dr;
    double ea = eps * b * (b - 2.0);
    ea = ea + eps;
    e.e = ea * .5;
    e.pad = 0;
    int si = atomicAdd(&sc->ev_count[h], 1);
    if (si < kNoallocEvCap) {
      e.sign = 1;
      sc->ev[(size_t)h * kNoallocEvCap + si] = e;
    } else if (atomicCAS(&sc->error, 0, DML_E_EVENT_OVERFLOW) == 0) {
      sc->err_info = h;
    }
    int sj = atomicAdd(&sc->ev_count[j], 1);
    if (sj < kNoallocEvCap) {
      e.sign = -1;
      sc->ev[(size_t)j * kNoallocEvCap + sj] = e;
    } else if (atomicCAS(&sc->error, 0, DML_E_EVENT_OVERFLOW) == 0) {
      sc->err_info = j;
    }
  }
}

// Ordered sums: hs%ref members start from zero, other atoms add to the
// caller's values (fuerza zeroes only hs%ref, dana.F90:1067-1073).
// A call whose pair kernel or member marks raised an error writes nothing.
__global__ void noalloc_sum_kernel(NoallocScratch* sc, int n_atoms, double* force, double* epot) {
  DML_GRID_WAIT();
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n_atoms) return;
  if (*(volatile int*)&sc->error != 0) return;
  int cnt = sc->ev_count[s];
  bool inref = sc->is_ref[s] != 0;
  if (!inref && cnt == 0) return;
  if (cnt > kNoallocEvCap) cnt = kNoallocEvCap;
  double fx, fy, fz, ep;
  if (inref) {
    fx = fy = fz = ep = 0.0;
  } else {
    fx = force[3 * s];
    fy = force[3 * s + 1];
    fz = force[3 * s + 2];
    ep = epot[s];
  }
  const dml::EvRec* ev = sc->ev + (size_t)s * kNoallocEvCap;
  unsigned char idx[kNoallocEvCap];
  unsigned long long keys[kNoallocEvCap];
  for (int i = 0; i < cnt; ++i) {
    unsigned long long kk = ev[i].key;
    int q = i;
    while (q > 0 && keys[q - 1] > kk) {
      keys[q] = keys[q - 1];
      idx[q] = idx[q - 1];
      --q;
    }
    keys[q] = kk;
    idx[q] = (unsigned char)i;
  }
  for (int q = 0; q < cnt; ++q) {
    const dml::EvRec& e = ev[idx[q]];
    if (e.sign > 0) {
      fx = fx + e.fx;
      fy = fy + e.fy;
      fz = fz + e.fz;
    } else {
      fx = fx - e.fx;
      fy = fy - e.fy;
      fz = fz - e.fz;
    }
    ep = ep + e.e;
  }
  force[3 * s] = fx;
  force[3 * s + 1] = fy;
  force[3 * s + 2] = fz;
  epot[s] = ep;
}

__global__ void noalloc_ref_mark_kernel(NoallocScratch* sc, const int32_t* ref, int n_ref,
                                        int n_atoms) {
  DML_GRID_WAIT();
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_ref) return;
  int h = ref[i];
  if (h < 0 || h >= n_atoms) {
    if (atomicCAS(&sc->error, 0, DML_E_ARG) == 0) sc->err_info = i;
    return;
  }
  sc->is_ref[h] = 1;
}

}  // namespace

extern "C" int dml_force_noalloc(const dml_params* prm, int32_t n_atoms, const double* pos,
                                 const int32_t* z, int32_t n_ref, const int32_t* ref,
                                 const int32_t* nn, const int32_t* list, int32_t ld,
                                 double* force, double* epot, void* stream) {
  if (!prm || !pos || !z || !force || !epot || (n_ref > 0 && (!ref || !nn || !list)))
    return DML_E_ARG;
  if (n_atoms < 0 || n_ref < 0 || n_ref > n_atoms || ld < 0) return DML_E_ARG;
  if (n_atoms > kNoallocMaxAtoms) return DML_E_CAPACITY;  // fixed scratch size
  if (n_atoms == 0) return 0;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return DML_E_CUDA;
  NoallocScratch* sc = nullptr;
  {
    // Once per device: the array's device address (its name is only a
    // host-side stand-in in host code).
    std::lock_guard<std::mutex> lk(g_addr_mu);
    if (!g_addr[dev]) {
      void* a = nullptr;
      if (cudaGetSymbolAddress(&a, g_noalloc_scratch) != cudaSuccess) return DML_E_CUDA;
      g_addr[dev] = (NoallocScratch*)a;
    }
    sc = g_addr[dev];
  }
  NoallocParams p;
  for (int k = 0; k < 2; ++k) {
    p.box[k] = prm->box[k];
    p.halfbox[k] = prm->box[k] * .5;
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double r0 = prm->r0[i][j], eps = prm->eps[i][j];
      double x2 = r0 * r0, x4 = x2 * x2;
      p.eps[i][j] = eps;
      p.r0sq[i][j] = r0 * r0;
      p.b0[i][j] = x2 * x4;
      p.c0[i][j] = eps * 12.0 * p.b0[i][j];
    }
  cudaStream_t s = (cudaStream_t)stream;
  const int B = 256;
  noalloc_clear_kernel<<<(n_atoms + B - 1) / B, B, 0, s>>>(sc, n_atoms);
  if (n_ref > 0) {
    noalloc_ref_mark_kernel<<<(n_ref + B - 1) / B, B, 0, s>>>(sc, ref, n_ref, n_atoms);
    noalloc_pairs_kernel<<<(n_ref + 7) / 8, B, 0, s>>>(sc, p, n_atoms, n_ref, pos, z, ref, nn,
                                                       list, ld);
  }
  noalloc_sum_kernel<<<(n_atoms + B - 1) / B, B, 0, s>>>(sc, n_atoms, force, epot);
  if (cudaGetLastError() != cudaSuccess) return DML_E_CUDA;
  int err = 0;
  if (cudaMemcpyAsync(&err, &sc->error, sizeof err, cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return DML_E_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return DML_E_CUDA;
  return err;
}
