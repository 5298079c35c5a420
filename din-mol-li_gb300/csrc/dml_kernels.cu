// dml_kernels.cu - sm_103a kernels of the plain FP64 form.
//
// Compiled with --fmad=false: no multiply-add is contracted, and every
// expression is written in the reference's evaluation order, so each kernel
// reproduces the serial reference bit for bit (double add, multiply, divide
// and sqrt are IEEE round-to-nearest on the device as on the host).
//
// Where work can be skipped without changing a bit of the result it is
// skipped: list entries are pre-filtered with FP32 distances carrying a
// rigorous error margin (the FP64 test decides every entry near a cut-off),
// and entries whose pair epsilon is zero add signed zeros, which leave a sum
// started at +0 unchanged.
#include <cuda_runtime.h>

#include <climits>

#include "../../include/dml_rng.h"
#include "dml_internal.h"

namespace dml {

namespace {

// The 27-cell stencil map of the linked cells (Cells.F90:28-36): offset of
// cell q along axis k in {-1, 0, 1}, packed as 2 bits (offset + 1) per cell
// in immediates, so that lanes asking for different cells read no memory
// (a constant-bank read with lane-dependent addresses serializes).
__device__ __forceinline__ int map_off(int q, int k) {
  const unsigned long long w = k == 0 ? 0x19090904686869ull
                               : k == 1 ? 0x10101016a6a6a5ull
                                        : 0xaa55aa80155ull;
  return (int)((w >> (2 * q)) & 3ull) - 1;
}

// Stencil index of the cell at offset (o1, o2, o3) in {-1, 0, 1}^3: the
// inverse of map_off, entry (o1 + 1) * 9 + (o2 + 1) * 3 + o3 + 1, 5 bits each.
__device__ __forceinline__ int map_inv(int o1, int o2, int o3) {
  const int i = (o1 + 1) * 9 + (o2 + 1) * 3 + o3 + 1;
  const unsigned long long w = i < 12 ? 0xa430c2224eb4df7ull
                               : i < 24 ? 0x484b58e5633b41aull
                                        : 0x2846ull;
  return (int)((w >> (5 * (i % 12))) & 31ull);
}

__device__ __forceinline__ void raise_error(Global* g, int code, int info) {
  if (atomicCAS(&g->error, 0, code) == 0) g->err_info = info;
}

__device__ __forceinline__ unsigned long long* u64(unsigned long long* p) { return p; }

__device__ __forceinline__ void count_add(unsigned long long* c, unsigned long long v) {
  atomicAdd(c, v);
}

// Conversions between binary64 and binary32 (round to nearest even; the
// widening is exact).  Both issue on GB300's narrow FP64 pipe, one
// instruction per value: a formulation on the integer pipes measured the same
// step time, because the compiler predicates its hardware fallback for the
// rare operands outside the normal range, which then issues all the same.
__device__ __forceinline__ float f64_to_f32_rn(double x) { return __double2float_rn(x); }

__device__ __forceinline__ double f32_to_f64(float f) { return (double)f; }

// a < b for binary64 values on the integer pipes (IEEE comparison: false
// with a NaN, -0 equal to +0): sign-magnitude mapped to two's complement.
__device__ __forceinline__ bool f64_lt(double a, double b) {
  long long x = __double_as_longlong(a), y = __double_as_longlong(b);
  const long long inf = 0x7FF0000000000000LL, mag = 0x7FFFFFFFFFFFFFFFLL;
  if ((x & mag) > inf || (y & mag) > inf) return false;
  x = x >= 0 ? x : LLONG_MIN - x;
  y = y >= 0 ? y : LLONG_MIN - y;
  return x < y;
}

// The deletion walk's pick (dana.F90:686-690), m = int(upick * n) + 1 capped
// at n, with upick = k * 2^-53 (k < 2^53) and n >= 0, exactly as the binary64
// product rounds: k * n (up to 84 bits) rounded to nearest even at 53
// significant bits, then scaled by 2^-53 (exact) and truncated.
__host__ __device__ inline int gcmc_pick_index(unsigned long long k, int n) {
  if (n <= 0) return n < 0 ? n : 0;
  const unsigned long long un = (unsigned long long)n;
  const unsigned long long lo = k * un;
#if defined(__CUDA_ARCH__)
  const unsigned long long hi = __umul64hi(k, un);
#else
  const unsigned long long hi = (unsigned long long)(((unsigned __int128)k * un) >> 64);
#endif
#if defined(__CUDA_ARCH__)
  const int len = hi ? 128 - __clzll((long long)hi) : (lo ? 64 - __clzll((long long)lo) : 0);
#else
  const int len = hi ? 128 - __builtin_clzll(hi) : (lo ? 64 - __builtin_clzll(lo) : 0);
#endif  // bit length of k * n
  unsigned long long q = 0;  // int(RN53(k n) / 2^53)
  if (len > 53) {
    const int sft = len - 53;  // 1 .. 31
    unsigned long long top = (lo >> sft) | (hi << (64 - sft));
    const unsigned long long r = lo & ((1ull << sft) - 1ull), half = 1ull << (sft - 1);
    if (r > half || (r == half && (top & 1ull))) top += 1ull;
    q = top >> (53 - sft);
  }
  const long long m = (long long)q + 1;
  return m > n ? n : (int)m;
}

// FP32 copy of a position; w carries the element as integer bits (0 for a
// slot that is not live), so reading it needs no conversion instruction.
__device__ __forceinline__ float4 to_f4(double4 p, int typ) {
  return make_float4(f64_to_f32_rn(p.x), f64_to_f32_rn(p.y), f64_to_f32_rn(p.z),
                     __int_as_float(typ));
}

__device__ __forceinline__ int elem_of(float4 q) { return __float_as_int(q.w); }

__device__ __forceinline__ double dot3(double x, double y, double z) {
  // dot_product as the reference evaluates it: ((0 + x*x) + y*y) + z*z.
  return (x * x + y * y) + z * z;
}

// x^6 = x^2 * x^4 and x^7 = (x * x^2) * x^4 (square-and-multiply), the
// evaluation of dana.F90:1117-1120 pinned by the reference's Ermak golden.
__device__ __forceinline__ double pow6(double x) {
  double x2 = x * x;
  double x4 = x2 * x2;
  return x2 * x4;
}
__device__ __forceinline__ double pow7(double x) {
  double x2 = x * x;
  double x3 = x * x2;
  double x4 = x2 * x2;
  return x3 * x4;
}

// vdistance (Groups.F90:995-1016): a - b, minimum image by idnint (round half
// away from zero) in x and y; z is not periodic.
__device__ __forceinline__ void vdist_nint(const RepConst& R, double4 a, double4 b, double& x,
                                           double& y, double& z) {
  x = a.x - b.x;
  y = a.y - b.y;
  z = a.z - b.z;
  x = x - R.box[0] * round(x * R.one_box[0]);
  y = y - R.box[1] * round(y * R.one_box[1]);
}

// FP32 pre-filter distance: minimum image by compare and add (no rounding
// or conversion instruction; on GB300 those issue on the narrow FP64 pipe).
// Near half a box the chosen image may differ from the exact one, where both
// images are farther than any cut-off.
__device__ __forceinline__ void vdist_nint_f(const RepConst& R, float4 a, float4 b, float& x,
                                             float& y, float& z) {
  x = a.x - b.x;
  y = a.y - b.y;
  z = a.z - b.z;
  if (x > R.halfboxf[0]) x -= R.boxf[0]; else if (x < -R.halfboxf[0]) x += R.boxf[0];
  if (y > R.halfboxf[1]) y -= R.boxf[1]; else if (y < -R.halfboxf[1]) y += R.boxf[1];
}

// int(x) + 1 for a cell index, with the x86-64 reference semantics: NaN or
// out-of-range values give the integer indefinite, i.e. an invalid index.
__device__ __forceinline__ int cell_index(double x, double cell) {
  double q = x / cell;
  if (!(q > -2147483649.0 && q < 2147483648.0)) return INT_MIN;
  return (int)q + 1;
}

// int(x / cell) + 1 estimated from the FP32 copy of the coordinate (the
// FP64 division issues on GB300's narrow FP64 pipe).  With xf = RN32(x) and
// inv = RN32(1/cell) the FP32 quotient q is within 3 * 2^-24 |q| of x/cell,
// so when q lies farther than 4e-7 q + 1e-6 from every integer, int(x/cell)
// = floor(q) exactly; for -0.999 < q <= 0 the true quotient lies in (-1, 0]
// (|q| < 1, error below 2e-7), where int() gives 0; otherwise kCellUndecided
// asks for cell_index.  The integer comes from adding 1.5 * 2^23 (round to
// nearest, FP32 adds only).
constexpr int kCellUndecided = INT_MIN + 1;
__device__ __forceinline__ int cell_index_est(float xf, float inv) {
  const float M = 12582912.0f;
  float q = xf * inv;
  float r = (q + M) - M;
  float dq = fabsf(q - r);
  if (q > 0.0f && q < 4194304.0f && dq > 4e-7f * q + 1e-6f)
    return (__float_as_int((q - 0.5f) + M) - 0x4B400000) + 1;
  // x/cell in (-1, 0] (coordinates on the lower box faces): int() truncates to 0
  if (q <= 0.0f && q > -0.999f) return 1;
  return kCellUndecided;
}

// Cell indices of a point from its FP32 and (when needed) FP64 coordinates.
__device__ __forceinline__ void cell_index3(const RepConst& R, float4 Pf, const double4* P,
                                            int& c1, int& c2, int& c3) {
  c1 = cell_index_est(Pf.x, R.inv_cellf[0]);
  c2 = cell_index_est(Pf.y, R.inv_cellf[1]);
  c3 = cell_index_est(Pf.z, R.inv_cellf[2]);
  if (c1 == kCellUndecided || c2 == kCellUndecided || c3 == kCellUndecided) {
    double4 Q = *P;
    if (c1 == kCellUndecided) c1 = cell_index(Q.x, R.cell[0]);
    if (c2 == kCellUndecided) c2 = cell_index(Q.y, R.cell[1]);
    if (c3 == kCellUndecided) c3 = cell_index(Q.z, R.cell[2]);
  }
}

// cgroup_sort_atom's range test (Cells.F90:289-294): 0 <= int(x/cell)+1 <=
// ncells+1 in every dimension, NaN out of range.  The quotient is formed only
// for coordinates within 1e-9 relative of a bound; elsewhere the bounds
// -2*cell < x < (ncells+1)*cell decide the same question.
__device__ __forceinline__ bool coord_in_tess(double x, double cell, int n) {
  double lo = -2.0 * cell, hi = (double)(n + 1) * cell;
  double tol = 1e-9 * (hi - lo);
  if (x > lo + tol && x < hi - tol) return true;
  if (!(x > lo - tol && x < hi + tol)) return false;  // far out, or NaN
  int c = cell_index(x, cell);
  return c >= 0 && c <= n + 1;
}

__device__ __forceinline__ bool in_tessellation(const RepConst& R, double4 P) {
  return coord_in_tess(P.x, R.cell[0], R.ncells[0]) && coord_in_tess(P.y, R.cell[1], R.ncells[1]) &&
         coord_in_tess(P.z, R.cell[2], R.ncells[2]);
}

// Prefix of the replicas' rows in use (one block): the warp-per-row kernels
// walk only the rows in use, the capacity headroom of every replica skipped.
__global__ void rank_prefix_kernel(Dev d) {
  DML_GRID_WAIT();
  __shared__ int ws[32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int base = 0; base < d.nrep; base += blockDim.x) {
    int i = base + threadIdx.x;
    int v = i < d.nrep ? d.sc[i].n_rank : 0, x = v;
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) ws[wid] = x;
    __syncthreads();
    if (wid == 0) {
      int w = lane < (int)(blockDim.x >> 5) ? ws[lane] : 0;
      for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      ws[lane] = w;
    }
    __syncthreads();
    int pre = (wid > 0 ? ws[wid - 1] : 0) + x - v;
    if (i < d.nrep) d.rank_pre[i] = carry + pre;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry += pre + v;
    __syncthreads();
  }
  if (threadIdx.x == 0) d.rank_pre[d.nrep] = carry;
}

// Rank (position in ref) of row i of the rows counted by the prefix `pre`
// over replicas (rank_pre: the rows in use; reb_pre: those of the replicas
// that rebuild).  A replica with no rows shares its prefix with the next
// one, so the largest replica whose first row is <= i owns row i.
__device__ __forceinline__ int row_rank_in(const Dev& d, const int* pre, int i) {
  int lo = 0, hi = d.nrep - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (__ldg(pre + mid) <= i) lo = mid; else hi = mid - 1;
  }
  return d.rc[lo].base + (i - __ldg(pre + lo));
}

__device__ __forceinline__ int row_rank(const Dev& d, int i) { return row_rank_in(d, d.rank_pre, i); }

// Per-position kernels: a block of kBlock threads covers kSpan consecutive
// positions (kSlotU per thread, kBlock apart, so each load instruction of a
// warp stays coalesced).  Replica capacities are multiples of kSpan, so a
// block lies inside one replica and loads that replica's constants and live
// counts once for all its positions.
__device__ __forceinline__ int block_rep(const Dev& d) { return d.rep_of[blockIdx.x * kSpan]; }
__device__ __forceinline__ int span_pos(int u) {
  return blockIdx.x * kSpan + u * kBlock + (int)threadIdx.x;
}

// The per-atom kernels whose result does not depend on the order of
// hs%ref (the integrators, ermak_b, the force scan, the capture commit and
// overlap_moveback's member count) walk hs slots instead of ranks: a slot
// belongs to hs%ref exactly when its rank is set.  Ranks follow the
// reference's attachment order, which GCMC insertions (appended, into the
// first free slots) decorrelate from slot order; slot order keeps the
// per-atom loads coalesced as the run goes on.
__device__ __forceinline__ int ref_slot(const Dev& d, int s, int end) {
  return s < end && d.rank[s] >= 0 ? s : -1;
}

__device__ __forceinline__ int warp_id_global() {
  return (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
}

// ----------------------------------------------------------------- step
// A new step: the counter, the displacement bound delta of this step's
// overlap search, and whether its near lists still need a search of their
// own (always with the Brownian integrator, which has no force scan).
__global__ void step_begin_kernel(Dev d, int near_stale) {
  DML_GRID_WAIT();
  Global* g = d.g;
  if (threadIdx.x == 0) {
    g->step += 1;
    g->delta2f_bits = 0u;
    g->chunk_event = 0;
    g->near_stale = near_stale;
    // overlap_moveback's counters (reset per call in the standalone path)
    g->again = 0;
    g->n_comp = 0;
    g->comp_total = 0;
    g->passes = 1;
  }
  for (int r = threadIdx.x; r < d.nrep; r += blockDim.x) {
    d.sc[r].passes = 1;
    d.sc[r].again2 = 0;
    d.pr_cnt[r * kCntStride + kCntAct] = 0;
  }
}

// The integrators' share of overlap_moveback in a fused step: the
// component state of the moving atom, and delta bounded from the FP32
// positions (|x - RN32(x)| <= 2^-24 |x|; the near radius adds the margin).
// Returns the squared FP32 move as its bit pattern (non-negative floats
// order as their bit patterns), for block_max_to.
__device__ __forceinline__ unsigned overlap_prepare_atom(const Dev& d, const RepConst& R, int h,
                                                         float4 before, float4 after) {
  d.uf[h] = h;
  d.active[h] = 0;
  d.comp_size[h] = 0;
  d.comp_fill[h] = 0;
  float x, y, z;
  vdist_nint_f(R, after, before, x, y, z);
  float dd = x * x + y * y + z * z;
  if (!(dd == dd)) dd = 0.0f;  // a NaN position takes no part (and stops at test_update)
  return __float_as_uint(dd);
}

// Maximum of v over the block, one atomic per block into *dst (a per-warp
// atomic on one address serialises some 10^5 operations per launch in the
// L2).  Every thread of the block must call it.
__device__ __forceinline__ void block_max_to(unsigned v, unsigned* dst) {
  __shared__ unsigned s_max;
  if (threadIdx.x == 0) s_max = 0u;
  __syncthreads();
  v = __reduce_max_sync(0xffffffffu, v);
  if ((threadIdx.x & 31) == 0 && v) atomicMax(&s_max, v);
  __syncthreads();
  if (threadIdx.x == 0 && s_max) atomicMax(dst, s_max);
}

// An atom whose element became F: listed for the capture commit.
__device__ __forceinline__ void note_f(const Dev& d, int h) {
  const int q = atomicAdd(&d.g->n_f, 1);
  if (q < d.cap) d.flist[q] = h;
}

// atom_pbc (dana.F90:1187-1250) on registers; returns true when deposited.
__device__ __forceinline__ bool atom_pbc_dev(const KParams& p, const RepConst& R, Scalars* sc,
                                             long long step,
                                             long long id, double* pp, double4& po, bool& po_changed,
                                             double4& vv, bool& v_changed, const double4& oc,
                                             int& typ, double zmax) {
  bool depos = false;
  double pox[2] = {po.x, po.y};
  for (int j = 0; j < 2; ++j) {
    if (pp[j] > R.box[j]) {
      pp[j] = pp[j] - R.box[j];
      pox[j] = pox[j] - R.box[j];
      po_changed = true;
    }
    if (pp[j] < 0.0) {
      pp[j] = pp[j] + R.box[j];
      pox[j] = pox[j] + R.box[j];
      po_changed = true;
    }
  }
  po.x = pox[0];
  po.y = pox[1];
  if (pp[2] > zmax) {
    if (p.integrator == DML_INTEGRATOR_ERMAK) {
      pp[2] = pp[2] - 2.0 * (pp[2] - zmax);
      vv.z = -vv.z;
      v_changed = true;
    } else {
      pp[0] = oc.x;
      pp[1] = oc.y;
      pp[2] = oc.z;
    }
  }
  if (pp[2] <= 0.0) {
    count_add(&sc->try_, 1ull);
    double ne = dml_uniform(dml_draw(R.seed, step, (uint64_t)id, DML_RNG_CAPTURE, 0));
    if (ne < p.prob) {
      count_add(&sc->depo, 1ull);
      typ = DML_Z_F;
      depos = true;
    }
    pp[0] = oc.x;
    pp[1] = oc.y;
    pp[2] = oc.z;
  }
  return depos;
}

// Box-Muller pair of the chosen form: the same two words as
// dml_normal_pair32f, the transform from the hardware's approximate
// log2, sin and cos (__log2f, __sinf, __cosf) instead of the exactly
// rounded series the plain form shares with the oracle.  u1 = (a + 1) 2^-32
// enters as 2^e m, e = -1 - clz(a + 1) and m in [1, 2) from the next 23
// bits (truncated), so no conversion instruction is needed and the radius
// still reaches the plain form's 6.66 sigma; u2 takes the top 23 bits of b.
// The approximate log2 is good to about 2^-22 absolute, so the normals agree
// with the plain form's within about 2e-6 (1 + r) for radii r above 0.05
// (the radius of the smaller ones, a fraction 1e-3 of the pairs, within 1e-3).
__device__ __forceinline__ void normal_pair_fast(uint32_t a, uint32_t b, float& n0, float& n1) {
  const uint32_t x = a + 1u;  // 0 stands for 2^32 (u1 = 1)
  float l2 = 0.0f;            // log2(u1)
  if (x != 0u) {
    const int lz = __clz((int)x);
    const uint32_t m = (x << lz) << 1;  // the bits after the leading one
    l2 = __log2f(__uint_as_float(0x3F800000u | (m >> 9))) + dml_small_i2f(-1 - lz);
  }
  const float r = __fsqrt_rn(-1.3862944f * l2);  // sqrt(-2 ln u1) = sqrt(-2 ln2 log2 u1)
  const float th = 6.2831853f * (__uint_as_float(0x3F800000u | (b >> 9)) - 1.0f);
  float sn, cs;
  __sincosf(th, &sn, &cs);
  n0 = r * cs;
  n1 = r * sn;
}

// The chosen form's FP32 velocity (first half) and acceleration (second
// half) of an atom's vel slot.
__device__ __forceinline__ void ldva(const double4* vel, int h, float4& v, float4& a) {
  const float4* q = reinterpret_cast<const float4*>(vel + h);
  v = q[0];
  a = q[1];
}
__device__ __forceinline__ void stv(double4* vel, int h, float x, float y, float z) {
  *reinterpret_cast<float4*>(vel + h) = make_float4(x, y, z, 0.0f);
}
__device__ __forceinline__ void stva(double4* vel, int h, float vx, float vy, float vz, float ax,
                                     float ay, float az) {
  float4* q = reinterpret_cast<float4*>(vel + h);
  q[0] = make_float4(vx, vy, vz, 0.0f);
  q[1] = make_float4(ax, ay, az, 0.0f);
}

// No atom_pbc action (wrap when x > box or x < 0, mirror when z > zmax,
// capture when z <= 0) can apply to a position whose FP32 copy f = RN32(x)
// satisfies 0 < f < RN32(bound) in every test: rounding to nearest is
// monotone, so x >= bound gives f >= RN32(bound) and x <= 0 gives f <= 0.
// boxf and zmaxf are RN32 of the FP64 bounds; a NaN is never quiet.
__device__ __forceinline__ bool pbc_quiet(const KParams& p, const RepConst& R, float4 f,
                                          float zmaxf) {
  return f.x > 0.0f && f.x < R.boxf[0] && f.y > 0.0f && f.y < R.boxf[1] && f.z > 0.0f &&
         f.z < zmaxf;
}

// ermak_a of the chosen form: each coordinate's increment (about 1e-2 Å per
// step) is formed in FP32 from the FP32 velocity, acceleration and noise and
// added to the FP64 position; atom_pbc runs in FP64 for the atoms near a
// wall, the box edge or the capture plane, as in the plain form.
// One atom's inputs to the chosen form's ermak_a, all loads issued together.
struct ErmIn {
  double2 Pxy;
  double Pz;
  float4 V, A, before;
  long long id;
  int typ;
};
__device__ __forceinline__ void erm_load(const Dev& d, int h, ErmIn& in) {
  in.Pxy = reinterpret_cast<const double2*>(d.pos + h)[0];
  in.Pz = reinterpret_cast<const double*>(d.pos + h)[2];
  ldva(d.vel, h, in.V, in.A);
  in.typ = d.typ[h];
  in.id = d.id[h];
  in.before = d.posf[h];
}
__device__ __forceinline__ unsigned ermak_a_mixed_atom(const Dev& d, const KParams& p,
                                                       const RepConst& R, Scalars* sc, int h,
                                                       const ErmIn& in, long long step,
                                                       double zmax, float zmaxf) {
  const double4 P = make_double4(in.Pxy.x, in.Pxy.y, in.Pz, 0.0);
  const float4 V = in.V, A = in.A;
  int typ = in.typ;
  const long long id = in.id;
  const float rf = p.rfacf[typ - 1], vf = p.vfacf[typ - 1];
  // six normals: both pairs of the first draw, the first pair of the second
  float nq[6];
  const dml_u4 w0 = dml_draw(R.seed, step, (uint64_t)id, DML_RNG_ERMAK, 0);
  const dml_u4 w1 = dml_draw(R.seed, step, (uint64_t)id, DML_RNG_ERMAK, 1);
  normal_pair_fast(w0.w[0], w0.w[1], nq[0], nq[1]);
  normal_pair_fast(w0.w[2], w0.w[3], nq[2], nq[3]);
  normal_pair_fast(w1.w[0], w1.w[1], nq[4], nq[5]);
  const float vv[3] = {V.x, V.y, V.z}, aa[3] = {A.x, A.y, A.z};
  double pp[3] = {P.x, P.y, P.z};
  float rv[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const float r1 = nq[2 * j], r2 = nq[2 * j + 1];
    const float inc = p.cc1f * vv[j] + p.cc2hf * aa[j] + rf * r1;
    pp[j] = pp[j] + f32_to_f64(inc);
    rv[j] = vf * (p.crv1f * r1 + p.crv2f * r2);
  }
  const int typ0 = typ;
  const float4 before = in.before;
  float4 after = to_f4(make_double4(pp[0], pp[1], pp[2], 0.0), typ);
  bool depos = false, po_changed = false, v_changed = false;
  double4 po;
  if (!pbc_quiet(p, R, after, zmaxf)) {
    po = d.pos_old[h];
    double4 Vd = make_double4(V.x, V.y, V.z, 0.0);
    depos = atom_pbc_dev(p, R, sc, step, id, pp, po, po_changed, Vd, v_changed, P, typ, zmax);
    after = to_f4(make_double4(pp[0], pp[1], pp[2], 0.0), typ);
  }
  d.old_cg[h] = P;
  d.pos[h] = make_double4(pp[0], pp[1], pp[2], 0.0);
  d.posf[h] = after;
  d.ranvf[h] = make_float4(rv[0], rv[1], rv[2], 0.0f);
  const unsigned mv = overlap_prepare_atom(d, R, h, before, after);
  if (po_changed) {
    d.pos_old[h] = po;
    d.posf_old[h] = to_f4(po, 0);
  }
  if (v_changed) stv(d.vel, h, V.x, V.y, -V.z);  // the mirror at zmax reverses vz
  if (typ != typ0) {
    d.typ[h] = (int8_t)typ;
    if (typ == DML_Z_F) note_f(d, h);
  }
  if (!depos) d.skip[h] = 0;
  return mv;
}

// ermak_a (dana.F90:974-1028): one thread per hs%ref member; one kernel
// per form, so that each gets only the registers its own path needs.
template <bool MIXED>
__device__ __forceinline__ unsigned ermak_a_at(const Dev& d, const KParams& p, int rep, int h,
                                               long long step, double zmax, float zmaxf) {
  const RepConst& R = d.rc[rep];
  Scalars* sc = d.sc + rep;
  if (MIXED) return 0u;
  double4 P = d.pos[h];
  double4 V = d.vel[h];
  double4 A = d.acel[h];
  int typ = d.typ[h];
  long long id = d.id[h];
  double rf = p.rfac[typ - 1], vf = p.vfac[typ - 1];
  double pp[3] = {P.x, P.y, P.z};
  double vv[3] = {V.x, V.y, V.z};
  double aa[3] = {A.x, A.y, A.z};
  double rv[3];
  double nq[6];
  dml_normal_quad(dml_draw(R.seed, step, (uint64_t)id, DML_RNG_ERMAK, 0), &nq[0]);
  const dml_u4 w1 = dml_draw(R.seed, step, (uint64_t)id, DML_RNG_ERMAK, 1);
  dml_normal_pair32(w1.w[0], w1.w[1], &nq[4], &nq[5]);
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    double r1 = nq[2 * j], r2 = nq[2 * j + 1];
    double ranr = rf * r1;
    pp[j] = pp[j] + p.cc1 * vv[j] + p.cc2h * aa[j] + ranr;
    rv[j] = vf * (p.crv1 * r1 + p.crv2 * r2);
  }
  double4 po = d.pos_old[h];
  bool po_changed = false, v_changed = false;
  int typ0 = typ;
  bool depos = atom_pbc_dev(p, R, sc, step, id, pp, po, po_changed, V, v_changed, P, typ, zmax);
  double4 np = make_double4(pp[0], pp[1], pp[2], 0.0);
  const float4 before = d.posf[h], after = to_f4(np, typ);
  d.old_cg[h] = P;
  d.pos[h] = np;
  d.posf[h] = after;
  d.ranv[h] = make_double4(rv[0], rv[1], rv[2], 0.0);
  const unsigned mv = overlap_prepare_atom(d, R, h, before, after);
  if (po_changed) {
    d.pos_old[h] = po;
    d.posf_old[h] = to_f4(po, 0);
  }
  if (v_changed) d.vel[h] = V;
  if (typ != typ0) {
    d.typ[h] = (int8_t)typ;
    if (typ == DML_Z_F) note_f(d, h);
  }
  if (!depos) d.skip[h] = 0;
  return mv;
}

// The block's hs%ref entries are read first, all four at once, and the
// replica's scalars once.  The chosen form runs four blocks per SM (64
// registers) and loads each atom's inputs just before integrating it:
// measured on config 5, 0.200 ms per launch against 0.219 with the next
// atom's inputs loaded ahead at three blocks per SM (80 registers) and 0.294
// with both at four blocks per SM (spills).
template <bool MIXED>
__global__ void __launch_bounds__(kBlock, MIXED ? 4 : 3) ermak_a_kernel(Dev d, KParams p, int n_rank) {
  DML_GRID_WAIT();
  const int rep = block_rep(d);
  const int end = d.rc[rep].base + d.sc[rep].n_slots;
  if ((int)blockIdx.x * kSpan >= end) return;
  int h0 = ref_slot(d, span_pos(0), end);
  int h1 = ref_slot(d, span_pos(1), end);
  int h2 = ref_slot(d, span_pos(2), end);
  int h3 = ref_slot(d, span_pos(3), end);
  const long long step = d.g->step;
  const double zmax = d.sc[rep].zmax;
  const float zmaxf = (float)zmax;
  unsigned mv = 0u;  // largest squared move of the block's atoms (bits)
  if (!MIXED) {
#pragma unroll 1
    for (int u = 0; u < kSlotU; ++u) {
      if (h0 >= 0) mv = max(mv, ermak_a_at<MIXED>(d, p, rep, h0, step, zmax, zmaxf));
      h0 = h1; h1 = h2; h2 = h3;
    }
  } else {
    const RepConst& R = d.rc[rep];
    Scalars* sc = d.sc + rep;
#pragma unroll 1
    for (int u = 0; u < kSlotU; ++u) {
      ErmIn cur;
      if (h0 >= 0) {
        erm_load(d, h0, cur);
        mv = max(mv, ermak_a_mixed_atom(d, p, R, sc, h0, cur, step, zmax, zmaxf));
      }
      h0 = h1; h1 = h2; h2 = h3; h3 = -1;
    }
  }
  block_max_to(mv, &d.g->delta2f_bits);
}

// cbrownian_hs (dana.F90:798-846): one thread per hs%ref member; one kernel
// per form.
template <bool MIXED>
__device__ __forceinline__ unsigned brownian_at(const Dev& d, const KParams& p, int rep, int h,
                                                long long step, double zmax, float zmaxf) {
  const RepConst& R = d.rc[rep];
  Scalars* sc = d.sc + rep;
  double4 P = d.pos[h];
  int typ = d.typ[h];
  long long id = d.id[h];
  if (MIXED) {
    // chosen form: FP32 increments added to the FP64 position, FP32 velocity
    const float facf = P.z > p.dif_switch_z ? p.fac_scf : p.fac_seif;
    float nf[4];
    const dml_u4 w = dml_draw(R.seed, step, (uint64_t)id, DML_RNG_BROWN, 0);
    normal_pair_fast(w.w[0], w.w[1], nf[0], nf[1]);
    normal_pair_fast(w.w[2], w.w[3], nf[2], nf[3]);
    double pp[3] = {P.x, P.y, P.z};
    float vf[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const float inc = nf[j] * facf;
      pp[j] = pp[j] + f32_to_f64(inc);
      vf[j] = inc * p.inv_hf;
    }
    const int typ0 = typ;
    const float4 before = d.posf[h];
    float4 after = to_f4(make_double4(pp[0], pp[1], pp[2], 0.0), typ);
    bool depos = false, po_changed = false, v_changed = false;
    double4 po;
    if (!pbc_quiet(p, R, after, zmaxf)) {
      po = d.pos_old[h];
      double4 Vd = make_double4(vf[0], vf[1], vf[2], 0.0);
      depos = atom_pbc_dev(p, R, sc, step, id, pp, po, po_changed, Vd, v_changed, P, typ, zmax);
      after = to_f4(make_double4(pp[0], pp[1], pp[2], 0.0), typ);
    }
    d.old_cg[h] = P;
    d.pos[h] = make_double4(pp[0], pp[1], pp[2], 0.0);
    d.posf[h] = after;
    stv(d.vel, h, vf[0], vf[1], vf[2]);
    const unsigned mv = overlap_prepare_atom(d, R, h, before, after);
    if (po_changed) {
      d.pos_old[h] = po;
      d.posf_old[h] = to_f4(po, 0);
    }
    if (typ != typ0) {
    d.typ[h] = (int8_t)typ;
    if (typ == DML_Z_F) note_f(d, h);
  }
    if (!depos) d.skip[h] = 0;
    return mv;
  }
  double fac = P.z > p.dif_switch_z ? p.fac_sc : p.fac_sei;
  double nrm[4];
  dml_normal_quad(dml_draw(R.seed, step, (uint64_t)id, DML_RNG_BROWN, 0), nrm);
  double pp[3] = {P.x, P.y, P.z};
  double vv[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    double posold = pp[j];
    pp[j] = posold + nrm[j] * fac;
    vv[j] = (pp[j] - posold) / p.h;
  }
  double4 V = make_double4(vv[0], vv[1], vv[2], 0.0);
  double4 po = d.pos_old[h];
  bool po_changed = false, v_changed = false;
  int typ0 = typ;
  bool depos = atom_pbc_dev(p, R, sc, step, id, pp, po, po_changed, V, v_changed, P, typ, zmax);
  double4 np = make_double4(pp[0], pp[1], pp[2], 0.0);
  const float4 before = d.posf[h], after = to_f4(np, typ);
  d.old_cg[h] = P;
  d.pos[h] = np;
  d.posf[h] = after;
  d.vel[h] = V;
  const unsigned mv = overlap_prepare_atom(d, R, h, before, after);
  if (po_changed) {
    d.pos_old[h] = po;
    d.posf_old[h] = to_f4(po, 0);
  }
  if (typ != typ0) {
    d.typ[h] = (int8_t)typ;
    if (typ == DML_Z_F) note_f(d, h);
  }
  if (!depos) d.skip[h] = 0;
  return mv;
}

// hs%ref entries and the replica's scalars read first, as in ermak_a.
template <bool MIXED>
__global__ void __launch_bounds__(kBlock, 4) brownian_kernel(Dev d, KParams p, int n_rank) {
  DML_GRID_WAIT();
  const int rep = block_rep(d);
  const int end = d.rc[rep].base + d.sc[rep].n_slots;
  if ((int)blockIdx.x * kSpan >= end) return;
  int h0 = ref_slot(d, span_pos(0), end);
  int h1 = ref_slot(d, span_pos(1), end);
  int h2 = ref_slot(d, span_pos(2), end);
  int h3 = ref_slot(d, span_pos(3), end);
  static_assert(kSlotU == 4, "four hs%ref entries per thread");
  const long long step = d.g->step;
  const double zmax = d.sc[rep].zmax;
  const float zmaxf = (float)zmax;
  unsigned mv = 0u;
#pragma unroll 1
  for (int u = 0; u < kSlotU; ++u) {
    if (h0 >= 0) mv = max(mv, brownian_at<MIXED>(d, p, rep, h0, step, zmax, zmaxf));
    h0 = h1;
    h1 = h2;
    h2 = h3;
  }
  block_max_to(mv, &d.g->delta2f_bits);
}

// Union-find over hs slots (overlap components): path halving, union by
// smaller root; bounded loops report DML_E_OVERLAP_PASSES.
__device__ int uf_find(volatile int* uf, int x) {
  for (int it = 0; it < (1 << 22); ++it) {
    int px = uf[x];
    if (px == x) return x;
    int ppx = uf[px];
    if (ppx != px) atomicCAS((int*)&uf[x], px, ppx);
    x = px;
  }
  return -1;
}

__device__ void uf_union(Global* g, volatile int* uf, int a, int b) {
  for (int it = 0; it < (1 << 20); ++it) {
    a = uf_find(uf, a);
    b = uf_find(uf, b);
    if (a < 0 || b < 0) break;
    if (a == b) return;
    if (a < b) {
      int t = a;
      a = b;
      b = t;
    }
    if (atomicCAS((int*)&uf[a], a, b) == a) return;
  }
  raise_error(g, DML_E_OVERLAP_PASSES, -1);
}

// Near radius of overlap_moveback, rc + 2 delta in FP32 with margin (a
// superset of the pairs that can touch during the passes).
__device__ __forceinline__ float near_radius2(const Dev& d, const KParams& p, const RepConst& R) {
  float delta = sqrtf(__uint_as_float(d.g->delta2f_bits));
  float rnf = (p.rcf + 2.0f * delta) * 1.000001f + 4.0f * R.margin + 1e-3f;
  return rnf * rnf;
}

// ---------------------------------------------------------------- fuerza
// Pass 1: the hs%ref members' list rows are scanned with the FP32
// pre-filter and every possibly interacting entry (r <= r0 + margin,
// eps != 0, not CG-CG) is appended to a compact queue.
// On GB300 an FP64 instruction occupies the narrow FP64 pipe for the whole
// warp whatever its active lanes, so the exact FP64 work is done afterwards
// on the dense queue (force_exact_kernel), 32 entries per instruction.
// One warp-wide pass over 32 / L rows, L lanes each (the lanes of a row
// agree on rep, r, h; h < 0 for no row).  Every lane of the warp takes part.
// Pf and n are the row owner's FP32 position and list length.
template <bool NEAR, int L>
__device__ __forceinline__ bool force_scan_row(const Dev& d, const KParams& p, int rep, int r,
                                               int h, float4 Pf, int n, float flag_r2 = -1.0f) {
  // each lane keeps 4 entries in flight
  constexpr int U = 4, STEP = L * U;
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, sl = lane % L, sub = lane / L;
  const unsigned smask = (L == 32 ? FULL : ((1u << L) - 1u)) << (sub * L);
  const RepConst& R = d.rc[rep];
  // the element comes with the position (posf.w)
  const int k = h >= 0 ? elem_of(Pf) : 0;
  if (h < 0) n = 0;
  int nmax = n;
#pragma unroll
  for (int o = L; o < 32; o <<= 1) nmax = max(nmax, __shfl_xor_sync(FULL, nmax, o));
  if (nmax == 0) return false;  // every row of the warp is empty
  const int* row = d.list + (size_t)(h >= 0 ? h : 0) * p.mnb;
  // With NEAR the same pass records overlap_moveback's near entries (list
  // entries within rc + 2 delta, in list order) and unites their components.
  const float rn2 = NEAR ? near_radius2(d, p, R) : 0.0f;
  int* near = d.near + (size_t)(h >= 0 ? h : 0) * kNearCap;
  int ncnt = 0;
  bool any = false, flag = false;
  const unsigned lt = (1u << lane) - 1u;
  // The entries of the next batch are loaded while this batch's positions
  // are, so that a batch waits on one load latency instead of two.
  int jn[U];
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int jj = L * u + sl;
    jn[u] = jj < n ? __ldg(row + jj) : -1;
  }
  for (int base = 0; base < nmax; base += STEP) {
    int j[U];
    float4 Q[U];
#pragma unroll
    for (int u = 0; u < U; ++u) j[u] = jn[u];
#pragma unroll
    for (int u = 0; u < U; ++u) Q[u] = j[u] >= 0 ? d.posf[j[u]] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int jj = base + STEP + L * u + sl;
      jn[u] = jj < n ? __ldg(row + jj) : -1;
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      // one FP32 minimum-image distance serves both tests; the element of
      // a slot that is not live (limbo, Neighbor.F90:1089-1092) is 0
      const int m = elem_of(Q[u]);
      const bool live = j[u] >= 0 && m != 0;
      float df = 0.0f;
      if (live) {
        float fx = Pf.x - Q[u].x, fy = Pf.y - Q[u].y, fz = Pf.z - Q[u].z;
        if (fx > R.halfboxf[0]) fx -= R.boxf[0]; else if (fx < -R.halfboxf[0]) fx += R.boxf[0];
        if (fy > R.halfboxf[1]) fy -= R.boxf[1]; else if (fy < -R.halfboxf[1]) fy += R.boxf[1];
        df = fx * fx + fy * fy + fz * fz;
      }
      flag = flag || (live && df <= flag_r2);
      // fuerza: r <= r0 + margin, eps != 0, not CG-CG (signed zeros only)
      const bool cand = live && !(k == DML_Z_CG && m == DML_Z_CG) && p.pair_on[k - 1][m - 1] &&
                        df <= R.r0f_pref2[k - 1][m - 1];
      const unsigned bc = __ballot_sync(FULL, cand);
      if (bc) {
        int base_q = 0;
        if (lane == 0) base_q = atomicAdd(&d.g->n_cand, __popc(bc));
        base_q = __shfl_sync(FULL, base_q, 0);
        if (cand) {
          int q = base_q + __popc(bc & lt);
          if (q < p.cand_cap) d.cand[q] = make_int4(r, base + L * u + sl, h, j[u]);
        }
      }
      if (NEAR) {
        const bool inc = live && df <= rn2;
        const unsigned bal = __ballot_sync(FULL, inc) & smask;
        if (inc) {
          int pre = __popc(bal & lt);
          if (ncnt + pre < kNearCap) near[ncnt + pre] = j[u];
          if (m != DML_Z_CG) {
            uf_union(d.g, (volatile int*)d.uf, h, j[u]);
            d.active[j[u]] = 1;
          }
        }
        ncnt += __popc(bal);
        any = any || bal != 0;
      }
    }
  }
  if (NEAR && sl == 0 && h >= 0) {
    d.near_count[h] = ncnt > kNearCap ? -1 : ncnt;
    if (any) d.active[h] = 1;
  }
  return flag;
}

// The rows in use, 32 / L per warp (L lanes each, so that the dependent
// loads of several rows overlap), by a fixed grid of warps; a row's rank
// comes from the replicas' prefix of rows in use.
template <bool NEAR, int L>
__global__ void __launch_bounds__(256) force_scan_kernel(Dev d, KParams p) {
  DML_GRID_WAIT();
  const int nw = gridDim.x * (blockDim.x >> 5);
  const int total = d.rank_pre[d.nrep];
  const int sub = (threadIdx.x & 31) / L;
  for (int w = warp_id_global(); (32 / L) * w < total; w += nw) {
    const int i = (32 / L) * w + sub;
    const int r = i < total ? row_rank(d, i) : 0;
    const int h = i < total ? d.ref[r] : -1;
    float4 Pf = make_float4(0.f, 0.f, 0.f, 0.f);
    int n = 0;
    if (h >= 0) {
      Pf = d.posf[h];
      n = d.nn[h];
    }
    force_scan_row<NEAR, L>(d, p, d.rep_of[r], r, h, Pf, n);
  }
}

// One lane per row: the hs slots of the replica's span, four per thread,
// their membership, positions and list lengths loaded up front.
template <bool NEAR>
__global__ void __launch_bounds__(kBlock) force_scan_span_kernel(Dev d, KParams p) {
  DML_GRID_WAIT();
  const int rep = block_rep(d);
  const int end = d.rc[rep].base + d.sc[rep].n_slots;
  if ((int)blockIdx.x * kSpan >= end) return;  // whole block: warps stay full
  static_assert(kSlotU == 4, "four rows per thread");
  // With short_scan a replica scans all its rows only at a full scan, which
  // flags the rows with an entry within sl_rs and lists them; between full
  // scans force_scan_listed_kernel walks the list instead.
  const bool short_mode = NEAR && p.short_scan;
  if (short_mode && !d.sc[rep].sl_mode) return;
  const float flag_r2 = short_mode ? d.sc[rep].sl_rs * d.sc[rep].sl_rs : -1.0f;
  int h0 = ref_slot(d, span_pos(0), end);
  int h1 = ref_slot(d, span_pos(1), end);
  int h2 = ref_slot(d, span_pos(2), end);
  int h3 = ref_slot(d, span_pos(3), end);
  const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
  float4 P0 = h0 >= 0 ? d.posf[h0] : z4, P1 = h1 >= 0 ? d.posf[h1] : z4;
  float4 P2 = h2 >= 0 ? d.posf[h2] : z4, P3 = h3 >= 0 ? d.posf[h3] : z4;
  int n0 = h0 >= 0 ? d.nn[h0] : 0, n1 = h1 >= 0 ? d.nn[h1] : 0;
  int n2 = h2 >= 0 ? d.nn[h2] : 0, n3 = h3 >= 0 ? d.nn[h3] : 0;
  const int lane = threadIdx.x & 31;
  // one copy of the row body, the rows rotated through registers
#pragma unroll 1
  for (int u = 0; u < kSlotU; ++u) {
    // the row's rank keys the reference's summation order of its entries
    const bool fl = force_scan_row<NEAR, 1>(d, p, rep, h0 >= 0 ? d.rank[h0] : 0, h0, P0, n0,
                                            flag_r2);
    if (short_mode) {
      if (h0 >= 0) d.rowflag[h0] = fl ? 1 : 0;
      const unsigned m = __ballot_sync(0xffffffffu, fl && h0 >= 0);
      if (m) {
        int b = 0;
        if (lane == __ffs(m) - 1) b = atomicAdd(&d.sl_nrows[rep], __popc(m));
        b = __shfl_sync(0xffffffffu, b, __ffs(m) - 1);
        if (fl && h0 >= 0)
          d.sl_rows[d.rc[rep].base + b + __popc(m & ((1u << lane) - 1u))] = h0;
      }
    }
    h0 = h1; h1 = h2; h2 = h3;
    P0 = P1; P1 = P2; P2 = P3;
    n0 = n1; n1 = n2; n2 = n3;
  }
}

// Between full scans (short_scan): the listed rows of the replicas scanned
// partially, each walked whole as the full scan walks it.  An unlisted row
// had no entry within sl_rs at the last full scan and no atom has moved by
// sl_disp since, so none of its entries can lie within the force pre-filter
// or the near radius now (its near count is still the 0 of that scan).
// Rows whose atom left hs%ref since (captures, deletions) are skipped.
template <bool NEAR>
__global__ void __launch_bounds__(kBlock) force_scan_listed_kernel(Dev d, KParams p) {
  DML_GRID_WAIT();
  const int total = d.sl_pre[d.nrep];
  const int nw = gridDim.x * (blockDim.x >> 5);
  const int lane = threadIdx.x & 31;
  for (int w = warp_id_global(); 32 * w < total; w += nw) {
    const int g = 32 * w + lane;
    int rep = 0, h = -1;
    if (g < total) {
      int lo = 0, hi = d.nrep - 1;  // the last replica whose prefix is <= g
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (d.sl_pre[mid] <= g) lo = mid; else hi = mid - 1;
      }
      rep = lo;
      h = d.sl_rows[d.rc[rep].base + g - d.sl_pre[rep]];
    }
    const int r = h >= 0 ? d.rank[h] : -1;
    if (r < 0) h = -1;
    const float4 P = h >= 0 ? d.posf[h] : make_float4(0.f, 0.f, 0.f, 0.f);
    const int n = h >= 0 ? d.nn[h] : 0;
    force_scan_row<NEAR, 1>(d, p, rep, r >= 0 ? r : 0, h, P, n);
  }
}

// A member's row that GCMC appends to between full force scans joins its
// replica's flagged-row list, once (the flag says it is listed).
__device__ __forceinline__ void flag_row(const Dev& d, int h) {
  if (atomicExch(&d.rowflag[h], 1) != 0) return;
  const int rep = d.rep_of[h];
  d.sl_rows[d.rc[rep].base + atomicAdd(&d.sl_nrows[rep], 1)] = h;
}

// An inserted atom's row: its slot was free, so no list holds it (slots are
// freed only by the list rebuilds, which make the next scan full) and it is
// listed whatever its stale flag says.
__device__ __forceinline__ void list_new_row(const Dev& d, int h) {
  atomicExch(&d.rowflag[h], 1);
  const int rep = d.rep_of[h];
  d.sl_rows[d.rc[rep].base + atomicAdd(&d.sl_nrows[rep], 1)] = h;
}

// Each replica's force scan mode for this step (KParams::short_scan), after
// the integrator: full when its lists changed or were loaded (sl_full), or
// when the displacement bound since its last full scan could bring an
// unflagged entry inside the larger of the force pre-filter and the near
// radius; otherwise flagged rows only.  delta is this step's largest move
// (the FP32 bound of ermak_a, plus margins); a full scan's flags are taken
// at this step's positions, which overlap_moveback may still move back by
// delta, so the bound restarts at delta.
__device__ int blk_scan_excl(int v, int* total);

__global__ void scan_mode_kernel(Dev d, KParams p) {
  DML_GRID_WAIT();
  const float delta = sqrtf(__uint_as_float(d.g->delta2f_bits));
  __shared__ int s_carry;
  if (threadIdx.x == 0) s_carry = 0;
  __syncthreads();
  for (int r0 = 0; r0 < d.nrep; r0 += blockDim.x) {
    const int r = r0 + threadIdx.x;
    int rows = 0;  // the listed rows this step walks (replicas scanned partially)
    if (r < d.nrep) {
      Scalars* sc = d.sc + r;
      const RepConst& R = d.rc[r];
      float f2 = 0.0f;
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
          if (p.pair_on[a][b]) f2 = fmaxf(f2, R.r0f_pref2[a][b]);
      const float need = fmaxf(sqrtf(near_radius2(d, p, R)), sqrtf(f2)) * 1.000001f;
      // delta comes from FP32 copies of the positions, each within half an
      // ulp of the coordinate (R.margin is 64 ulps of the largest one)
      const float dlt = (delta + 0.125f * R.margin) * 1.000001f;
      const float D = sc->sl_disp + dlt;
      if (sc->sl_full || need + 2.0f * D > sc->sl_rs) {
        sc->sl_mode = 1;
        sc->sl_full = 0;
        sc->sl_disp = dlt;
        sc->sl_rs = need + p.short_skin;
        d.sl_nrows[r] = 0;  // the full scan lists the flagged rows again
        sc->sl_nfull += 1;
      } else {
        sc->sl_mode = 0;
        sc->sl_disp = D;
        sc->sl_npartial += 1;
        rows = d.sl_nrows[r];
      }
    }
    int tot;
    const int e = blk_scan_excl(rows, &tot);
    if (r < d.nrep) d.sl_pre[r] = s_carry + e;
    __syncthreads();
    if (threadIdx.x == 0) s_carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) d.sl_pre[d.nrep] = s_carry;
}

// Every replica's next force scan is full (lists or positions changed outside
// the step sequence).
__global__ void scan_invalidate_kernel(Dev d) {
  DML_GRID_WAIT();
  for (int r = threadIdx.x; r < d.nrep; r += blockDim.x) d.sc[r].sl_full = 1;
}

// Exact FP64 evaluation of the queued entries (dana.F90:1095-1134), one
// thread per entry, recording each interacting entry for both atoms with the
// key (rank, jj) that orders the reference's accumulation.
__global__ void force_exact_kernel(Dev d, KParams p) {
  DML_GRID_WAIT();
  int nc = d.g->n_cand;
  if (nc > p.cand_cap) {
    if (blockIdx.x == 0 && threadIdx.x == 0) raise_error(d.g, DML_E_EVENT_OVERFLOW, nc);
    nc = p.cand_cap;
  }
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nc; q += gridDim.x * blockDim.x) {
    int4 c = d.cand[q];
    int r = c.x, jj = c.y, h = c.z, j = c.w;
    const RepConst& R = d.rc[d.rep_of[h]];
    int k = d.typ[h], m = d.typ[j];
    double4 Pi = d.pos[h], Pj = d.pos[j];
    double vx = Pi.x - Pj.x, vy = Pi.y - Pj.y, vz = Pi.z - Pj.z;
    if (vx > R.halfbox[0]) {
      vx = vx - R.box[0];
    } else if (vx < -R.halfbox[0]) {
      vx = vx + R.box[0];
    }
    if (vy > R.halfbox[1]) {
      vy = vy - R.box[1];
    } else if (vy < -R.halfbox[1]) {
      vy = vy + R.box[1];
    }
    double dr = dot3(vx, vy, vz);
    if (dr > p.r0sq[k - 1][m - 1]) continue;
    double eps = p.eps[k - 1][m - 1];
    dr = sqrt(dr);
    double cc = p.c0[k - 1][m - 1] / pow7(dr);
    double b = p.b0[k - 1][m - 1] / pow6(dr);
    double aux = cc * (b - 1.0);
    EvRec e;
    e.key = ((unsigned long long)(unsigned)r << 32) | (unsigned)jj;
    e.fx = aux * vx / dr;
    e.fy = aux * vy / dr;
    e.fz = aux * vz / dr;
    double ea = eps * b * (b - 2.0);
    ea = ea + eps;
    e.e = ea * .5;
    e.pad = 0;
    int si = atomicAdd(&d.ev_count[h], 1);
    if (si < p.ev_cap) {
      e.sign = 1;
      d.ev[(size_t)h * p.ev_cap + si] = e;
    } else {
      raise_error(d.g, DML_E_EVENT_OVERFLOW, h);
    }
    int sj = atomicAdd(&d.ev_count[j], 1);
    if (sj < p.ev_cap) {
      e.sign = -1;
      d.ev[(size_t)j * p.ev_cap + sj] = e;
    } else {
      raise_error(d.g, DML_E_EVENT_OVERFLOW, j);
    }
  }
}

// ermak_b (dana.F90:1031-1052) for one atom.
__device__ __forceinline__ void ermak_b_atom(const Dev& d, const KParams& p, int h, int typ,
                                             double4 F) {
  if (typ == DML_Z_CG) return;
  double m = p.mass[typ - 1];
  double4 V = d.vel[h], A = d.acel[h], R = d.ranv[h];
  V.x = p.cc0 * V.x + p.cc1mcc2 * A.x + p.cc2 * F.x / m + R.x;
  V.y = p.cc0 * V.y + p.cc1mcc2 * A.y + p.cc2 * F.y / m + R.y;
  V.z = p.cc0 * V.z + p.cc1mcc2 * A.z + p.cc2 * F.z / m + R.z;
  A.x = F.x / m;
  A.y = F.y / m;
  A.z = F.z / m;
  d.vel[h] = V;
  d.acel[h] = A;
}

// ermak_b of the mixed form: F/m as F * (1/m) (one FP64 multiply instead of
// a division; the FP64 divide is a long sequence on GB300's narrow FP64
// pipe), so the velocities differ from the plain form in the last bits.
// ermak_b of the chosen form (FP32 velocity side); the force arrives as
// FP32 (from the fixed-point sums), zero for the many atoms with no pair.
__device__ __forceinline__ void ermak_b_atom_mixed(const Dev& d, const KParams& p, int h, int typ,
                                                   float fx, float fy, float fz) {
  if (typ == DML_Z_CG) return;
  const float im = p.inv_massf[typ - 1];
  float4 V, A;
  ldva(d.vel, h, V, A);
  const float4 R = d.ranvf[h];
  const float ax = fx * im, ay = fy * im, az = fz * im;
  stva(d.vel, h, p.cc0f * V.x + p.cc1mcc2f * A.x + p.cc2f * ax + R.x,
       p.cc0f * V.y + p.cc1mcc2f * A.y + p.cc2f * ay + R.y,
       p.cc0f * V.z + p.cc1mcc2f * A.z + p.cc2f * az + R.z, ax, ay, az);
}

// Pass 2: one thread per hs slot sums its recorded entries in key order,
// i.e. in the reference's global accumulation order (hs%ref order x list
// order, with the Newton reaction applied to both atoms of every entry).
template <bool FUSE_B>
__device__ __forceinline__ void force_sum_at(Dev d, KParams p, int n_slots, int rep, int pos) {
  const RepConst& R = d.rc[rep];
  Scalars* sc = d.sc + rep;
  n_slots = R.base + sc->n_slots;  // positions in use end here
  const int s = pos;
  if (s == 0) d.g->n_cand = 0;
  if (s >= n_slots) return;
  if (d.state[s] != ST_LIVE) return;
  int cnt = d.ev_count[s];
  bool inref = d.rank[s] >= 0;
  if (!inref && cnt == 0) return;
  if (cnt > p.ev_cap) cnt = p.ev_cap;  // overflow already raised
  double4 F;
  double ep;
  if (inref) {
    F = make_double4(0.0, 0.0, 0.0, 0.0);
    ep = 0.0;
  } else {
    F = d.force[s];
    ep = d.epot[s];
  }
  if (cnt > 0) {
    const EvRec* ev = d.ev + (size_t)s * p.ev_cap;
    // order of entries: insertion sort of the keys (few entries per atom)
    unsigned char idx[128];
    unsigned long long keys[128];
    int c = cnt < 128 ? cnt : 128;
    if (cnt > 128) raise_error(d.g, DML_E_EVENT_OVERFLOW, s);
    for (int i = 0; i < c; ++i) {
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
    for (int q = 0; q < c; ++q) {
      const EvRec& e = ev[idx[q]];
      if (e.sign > 0) {
        F.x = F.x + e.fx;
        F.y = F.y + e.fy;
        F.z = F.z + e.fz;
      } else {
        F.x = F.x - e.fx;
        F.y = F.y - e.fy;
        F.z = F.z - e.fz;
      }
      ep = ep + e.e;
    }
    d.ev_count[s] = 0;
  }
  d.force[s] = F;
  d.epot[s] = ep;
  if (FUSE_B && inref) ermak_b_atom(d, p, s, d.typ[s], F);
}

template <bool FUSE_B>
__global__ void force_sum_kernel(Dev d, KParams p, int n_slots) {
  DML_GRID_WAIT();
  const int rep = block_rep(d);
#pragma unroll
  for (int u = 0; u < kSlotU; ++u) force_sum_at<FUSE_B>(d, p, n_slots, rep, span_pos(u));
}

__device__ __forceinline__ void ermak_b_at(Dev d, KParams p, int n_rank, int rep, int pos) {
  const RepConst& R = d.rc[rep];
  Scalars* sc = d.sc + rep;
  const int r = pos;
  if (r - R.base >= sc->n_rank) return;
  int h = d.ref[r];
  if (h < 0) return;
  if (p.mixed) {
    const double4 F = d.force[h];
    ermak_b_atom_mixed(d, p, h, d.typ[h], (float)F.x, (float)F.y, (float)F.z);
  } else
    ermak_b_atom(d, p, h, d.typ[h], d.force[h]);
}

__global__ void ermak_b_kernel(Dev d, KParams p, int n_rank) {
  DML_GRID_WAIT();
  const int rep = block_rep(d);
#pragma unroll
  for (int u = 0; u < kSlotU; ++u) ermak_b_at(d, p, n_rank, rep, span_pos(u));
}


// ------------------------------------------------------- mixed-precision force
// The chosen form of fuerza: the pair difference, the core (r0/r)^2,
// (r0/r)^6, (r0/r)^6 - 1 and the scalar force and energy are taken in FP64 (positions reach 350 Å, where an FP32
// coordinate has a 3e-5 Å ulp), the pair force and energy in FP32, and both
// are accumulated as int64 fixed point (2^32 per eV/Å and per eV).  Integer addition is associative, so the sums do not
// depend on the order of the atomics: deterministic without ordering.
__device__ __forceinline__ long long to_fixed(const KParams& p, float v, double scale) {
  double x = (double)v * scale;
  if (!(fabs(x) < 4.0e18)) return LLONG_MIN;  // overflow marker
  return __double2ll_rn(x);
}

// A slot's first pair of the call sets its bit and lists it (once).
__device__ __forceinline__ void touch_slot(const Dev& d, int h) {
  const unsigned bit = 1u << (h & 31);
  if (atomicOr(&d.ftouch[h >> 5], bit) & bit) return;
  d.ftlist[atomicAdd(&d.g->n_ftouch, 1)] = h;
}

__global__ void force_exact_mixed_kernel(Dev d, KParams p) {
  DML_GRID_WAIT();
  int nc = d.g->n_cand;
  if (nc > p.cand_cap) {
    if (blockIdx.x == 0 && threadIdx.x == 0) raise_error(d.g, DML_E_EVENT_OVERFLOW, nc);
    nc = p.cand_cap;
  }
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nc; q += gridDim.x * blockDim.x) {
    int4 c = d.cand[q];
    int h = c.z, j = c.w;
    const RepConst& R = d.rc[d.rep_of[h]];
    int k = d.typ[h], m = d.typ[j];
    double4 Pi = d.pos[h], Pj = d.pos[j];
    double dx = Pi.x - Pj.x, dy = Pi.y - Pj.y, dz = Pi.z - Pj.z;
    if (dx > R.halfbox[0]) dx -= R.box[0]; else if (dx < -R.halfbox[0]) dx += R.box[0];
    if (dy > R.halfbox[1]) dy -= R.box[1]; else if (dy < -R.halfbox[1]) dy += R.box[1];
    // The distance-dependent core, q = (r0/r)^2 and b = q^3, is formed in
    // FP64 and rounded once to FP32: the force goes as r^-14 in the core, so
    // FP32 roundings of r^2, 1/r^2 and q^3 would be amplified about sixfold.
    // The force polynomial, the vector and the energy are FP32.
    double r2d = dot3(dx, dy, dz);
    if (r2d > p.r0sq[k - 1][m - 1]) continue;
    // The scalars |F|/r = 12 eps b (b-1) / r^2 and half the pair energy
    // eps (b-1)^2 / 2 are formed from the FP64 core and rounded once (b - 1
    // before any rounding: near the cut-off b -> 1); the force vector is the
    // FP32 product of that scalar with the FP32 difference.
    double qd = p.r0sq[k - 1][m - 1] / r2d;
    double bd = qd * qd * qd;
    double bm1 = bd - 1.0;
    float fr = (float)(p.c12[k - 1][m - 1] * qd * (bd * bm1));
    float e = (float)(0.5 * p.eps[k - 1][m - 1] * (bm1 * bm1));
    float vx = (float)dx, vy = (float)dy, vz = (float)dz;
    long long fx = to_fixed(p, fr * vx, p.fix_scale);
    long long fy = to_fixed(p, fr * vy, p.fix_scale);
    long long fz = to_fixed(p, fr * vz, p.fix_scale);
    long long fe = to_fixed(p, e, p.fix_scale);
    if (fx == LLONG_MIN || fy == LLONG_MIN || fz == LLONG_MIN || fe == LLONG_MIN) {
      raise_error(d.g, DML_E_FIXEDPOINT_OVERFLOW, h);
      continue;
    }
    touch_slot(d, h);
    touch_slot(d, j);
    unsigned long long* ai = (unsigned long long*)(d.facc + 4 * (size_t)h);
    unsigned long long* aj = (unsigned long long*)(d.facc + 4 * (size_t)j);
    atomicAdd(ai + 0, (unsigned long long)fx);
    atomicAdd(ai + 1, (unsigned long long)fy);
    atomicAdd(ai + 2, (unsigned long long)fz);
    atomicAdd(ai + 3, (unsigned long long)fe);
    atomicAdd(aj + 0, (unsigned long long)(-fx));
    atomicAdd(aj + 1, (unsigned long long)(-fy));
    atomicAdd(aj + 2, (unsigned long long)(-fz));
    atomicAdd(aj + 3, (unsigned long long)fe);
  }
}

// Fixed point -> double, accumulators cleared, ermak_b fused.
//
// The sums are taken without a pass over every slot: forces of the chosen form
// are sparse (a pair inside r0 is rare between hard-core ions), so only the
// slots listed by force_exact_mixed_kernel read and clear their fixed-point
// accumulators (force_touched_kernel), and the hs%ref members (the only
// atoms whose force fuerza zeroes and ermak_b reads) are walked by rank
// (force_ref_kernel): a member with no pair gets force 0, epot 0 and
// ermak_b with a zero force, touching neither the accumulators nor the
// electrode slots.
template <bool FUSE_B>
__global__ void force_touched_kernel(Dev d, KParams p) {
  DML_GRID_WAIT();
  const int nt = d.g->n_ftouch;
  const double inv = p.fix_inv;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nt; q += gridDim.x * blockDim.x) {
    const int s = d.ftlist[q];
    long long* a = d.facc + 4 * (size_t)s;
    const long long ax = a[0], ay = a[1], az = a[2], ae = a[3];
    a[0] = 0;
    a[1] = 0;
    a[2] = 0;
    a[3] = 0;
    double4 F;
    double ep;
    const bool inref = d.rank[s] >= 0;
    if (inref) {
      F = make_double4((double)ax * inv, (double)ay * inv, (double)az * inv, 0.0);
      ep = (double)ae * inv;
    } else {  // fuerza adds to the atoms outside hs%ref
      F = d.force[s];
      F.x += (double)ax * inv;
      F.y += (double)ay * inv;
      F.z += (double)az * inv;
      ep = d.epot[s] + (double)ae * inv;
      atomicAnd(&d.ftouch[s >> 5], ~(1u << (s & 31)));
    }
    d.force[s] = F;
    d.epot[s] = ep;
    if (inref) atomicOr(&d.fnz[s >> 5], 1u << (s & 31));
    if (FUSE_B && inref) ermak_b_atom_mixed(d, p, s, d.typ[s], (float)F.x, (float)F.y, (float)F.z);
  }
}

template <bool FUSE_B>
__device__ __forceinline__ void force_ref_at(const Dev& d, const KParams& p, int rep, int s) {
  const int h = ref_slot(d, s, d.rc[rep].base + d.sc[rep].n_slots);
  if (h < 0) return;
  const unsigned bit = 1u << (h & 31);
  if (d.ftouch[h >> 5] & bit) {  // summed by force_touched_kernel
    atomicAnd(&d.ftouch[h >> 5], ~bit);
    return;
  }
  if (d.fnz[h >> 5] & bit) {  // zero where a force may stand; elsewhere it is zero already
    d.force[h] = make_double4(0.0, 0.0, 0.0, 0.0);
    d.epot[h] = 0.0;
    atomicAnd(&d.fnz[h >> 5], ~bit);
  }
  if (FUSE_B) ermak_b_atom_mixed(d, p, h, d.typ[h], 0.0f, 0.0f, 0.0f);
}

template <bool FUSE_B>
__global__ void force_ref_kernel(Dev d, KParams p) {
  DML_GRID_WAIT();
  const int rep = block_rep(d);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    d.g->n_cand = 0;
    d.g->n_ftouch = 0;
  }
  if ((int)blockIdx.x * kSpan >= d.rc[rep].base + d.sc[rep].n_slots) return;
#pragma unroll
  for (int u = 0; u < kSlotU; ++u) force_ref_at<FUSE_B>(d, p, rep, span_pos(u));
}

// ----------------------------------------------------------- test_update
// Top-2 merge on the bit patterns of non-negative doubles, which order like
// unsigned integers: the integer pipe gives the FP64 maximum exactly.
__device__ __forceinline__ void top2_merge(unsigned long long& a1, unsigned long long& a2,
                                           unsigned long long b1, unsigned long long b2) {
  unsigned long long hi = a1 > b1 ? a1 : b1;
  unsigned long long lo1 = a1 > b1 ? b1 : a1;
  unsigned long long lo2 = a2 > b2 ? a2 : b2;
  a1 = hi;
  a2 = lo1 > lo2 ? lo1 : lo2;
}

// do_pbc (Groups.F90:1440-1467) + inq_dispmax (Neighbor.F90:635-666) + the
// update decision (Neighbor.F90:697-710), sqrt(d1) + sqrt(d2) > skin with
// d1 >= d2 the two largest |pos - pos_old|^2 (exact FP64 in the reference).
//
// Most atoms need no FP64 here: an atom whose FP32 coordinates lie farther
// than the margin from 0 and the box edge (x, y) and from the tessellation
// bounds (z) is neither wrapped nor out of the tessellation, and its FP32
// displacement |posf - posf_old| is within the margin e of the exact one in
// sqrt space.  The FP32 top-2 F1 >= F2 then decides whenever sqrt(F1) +
// sqrt(F2) is farther than 4e from skin; otherwise the replica's last block
// takes the exact top-2 over the atoms with sqrt(rdf) >= sqrt(F2) - 3e (any
// atom of the exact top-2 qualifies) and decides in FP64 as the reference.
__device__ __forceinline__ double4 ldcg_d4(const double4* p) {
  const double2* q = reinterpret_cast<const double2*>(p);
  double2 a = __ldcg(q), b = __ldcg(q + 1);
  return make_double4(a.x, a.y, b.x, b.y);
}

__device__ __forceinline__ void top2f(float& a1, float& a2, float b1, float b2) {
  float hi = fmaxf(a1, b1), lo1 = fminf(a1, b1), lo2 = fmaxf(a2, b2);
  a1 = hi;
  a2 = fmaxf(lo1, lo2);
}

__device__ __forceinline__ float disp2f(float4 P, float4 O) {
  float x = P.x - O.x, y = P.y - O.y, z = P.z - O.z;
  return (x * x + y * y) + z * z;
}

__device__ __forceinline__ void decide_rebuild(const Dev& d, Scalars* sc, int rebuild) {
  sc->rebuild = rebuild;
  if (rebuild) {
    sc->sl_full = 1;  // new lists: the next force scan sets the row flags again
    sc->nupd += 1;
    sc->max_nn = 0;
    atomicOr(&d.g->any_rebuild, 1);
  }
}

// The step's second test_update (second = 1) follows overlap_moveback,
// which moves atoms back to their step-start positions and nothing else:
// a block none of whose atoms moved (dirty = 0) has the positions, wraps and
// displacements of the first test_update, so it reuses that call's FP32
// top-2 (or, in a replica whose list the first call rebuilt, pos_old = pos
// and every displacement is 0).  Dirty blocks are recomputed in full.
__global__ void __launch_bounds__(kBlock, 6) pbc_dispmax_kernel(Dev d, KParams p, int n_slots,
                                                                 int second) {
  DML_GRID_WAIT();
  // grids are sized by capacity; the block's replica gives the live count
  const int rep = block_rep(d);
  const RepConst& R = d.rc[rep];
  Scalars* sc = d.sc + rep;
  n_slots = R.base + sc->n_slots;  // positions in use end here
  // the spans in use take part (the first one always, so that every replica
  // decides); a block past them leaves at once
  const int b0 = R.base / kSpan;
  const int nu = max(1, (n_slots - R.base + kSpan - 1) / kSpan);
  if ((int)blockIdx.x - b0 >= nu) return;
  const float tinyf = 1e-16f;
  const float e = R.margin;
  float a1 = tinyf, a2 = tinyf;
  // The loads of all the thread's positions are issued together: a slot is
  // live exactly when its FP32 copy carries an element (w != 0; limbo and
  // free slots hold 0), so no state load has to come first.
  bool live[kSlotU];
  float4 Pfu[kSlotU], Ofu[kSlotU];
  bool used = (int)blockIdx.x * kSpan < n_slots;
  if (second && used && d.dirty[blockIdx.x] == 0) {
    used = false;  // nothing moved here since the first call
    if (threadIdx.x == 0 && !sc->rebuild) {
      a1 = __uint_as_float(d.part1[2 * blockIdx.x]);
      a2 = __uint_as_float(d.part1[2 * blockIdx.x + 1]);
    }
  }
  if (!second && threadIdx.x == 0) d.dirty[blockIdx.x] = 0;
#pragma unroll
  for (int u = 0; u < kSlotU; ++u) {
    const int s = span_pos(u);
    const bool in = used && s < n_slots;
    Pfu[u] = in ? d.posf[s] : make_float4(0.f, 0.f, 0.f, 0.f);
    Ofu[u] = in ? d.posf_old[s] : make_float4(0.f, 0.f, 0.f, 0.f);
    live[u] = in && elem_of(Pfu[u]) != 0;
  }
  // With rho_fused (piston), calc_rho's count of live atoms in (z0, zt) is
  // taken here: z changes only by the integrator, overlap_moveback (dirty
  // blocks) and the piston, which follows calc_rho, so the step's second call
  // has calc_rho's positions and a clean block keeps the first call's count.
  int cnt = 0;
  const double cz0 = sc->z0, czt = sc->zmax;
  if (p.rho_fused) {
    const float z0f = (float)cz0, ztf = (float)czt;
#pragma unroll
    for (int u = 0; u < kSlotU; ++u) {
      if (!live[u]) continue;
      const float zf = Pfu[u].z;  // z in (z0, zt) from the FP32 copy (monotone rounding)
      if (zf > z0f && zf < ztf) {
        cnt += 1;
      } else if (!(zf < z0f || zf > ztf)) {
        const double z = d.pos[span_pos(u)].z;
        cnt += (z > cz0 && z < czt) ? 1 : 0;
      }
    }
  }
#pragma unroll
  for (int u = 0; u < kSlotU; ++u) {
  const int s = span_pos(u);
  if (live[u]) {
    float4 Pf = Pfu[u], Of = Ofu[u];
    // no wrap (x >= box or x < 0, exact as in pbc_quiet; +0.0f rounds from
    // x in [0, 2^-150], which needs none) and inside the tessellation in x, y
    const bool sx = (Pf.x > 0.0f || __float_as_uint(Pf.x) == 0u) && Pf.x < R.boxf[0];
    const bool sy = (Pf.y > 0.0f || __float_as_uint(Pf.y) == 0u) && Pf.y < R.boxf[1];
    bool safe = sx && sy;
    if (safe && R.use_cells)
      safe = Pf.z > -2.0f * R.cellf[2] + e && Pf.z < R.tess_hif - e;
    if (!safe) {
      double4 P = d.pos[s];
      double4 O = d.pos_old[s];
      bool ch = false;
      if (P.x >= R.box[0]) {
        P.x = P.x - R.box[0];
        O.x = O.x - R.box[0];
        ch = true;
      } else if (P.x < 0.0) {
        P.x = P.x + R.box[0];
        O.x = O.x + R.box[0];
        ch = true;
      }
      if (P.y >= R.box[1]) {
        P.y = P.y - R.box[1];
        O.y = O.y - R.box[1];
        ch = true;
      } else if (P.y < 0.0) {
        P.y = P.y + R.box[1];
        O.y = O.y + R.box[1];
        ch = true;
      }
      if (ch) {
        d.pos[s] = P;
        d.pos_old[s] = O;
        Pf = to_f4(P, d.typ[s]);
        Of = to_f4(O, 0);
        d.posf[s] = Pf;
        d.posf_old[s] = Of;
      }
      // cgroup_sort runs at every test_update (Neighbor.F90:687-691) and
      // stops on an atom outside the tessellation (Cells.F90:293-294).
      if (R.use_cells && !in_tessellation(R, P)) raise_error(d.g, DML_E_OUT_OF_TESSELLATION, s);
    }
    float rdf = disp2f(Pf, Of);
    // a NaN displacement never passes `rd > dispmax` (Neighbor.F90:657-661)
    if (rdf == rdf) top2f(a1, a2, rdf, tinyf);
  }
  }
  for (int off = 16; off > 0; off >>= 1) {
    float b1 = __shfl_down_sync(0xffffffffu, a1, off);
    float b2 = __shfl_down_sync(0xffffffffu, a2, off);
    top2f(a1, a2, b1, b2);
    cnt += __shfl_down_sync(0xffffffffu, cnt, off);
  }
  __shared__ float w1[32], w2[32];
  __shared__ int wc[32];
  __shared__ unsigned long long x1[32], x2[32];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nwarp = blockDim.x >> 5;
  if (lane == 0) {
    w1[wid] = a1;
    w2[wid] = a2;
    wc[wid] = cnt;
  }
  __syncthreads();
  __shared__ bool last;
  if (threadIdx.x == 0) {
    float b1 = tinyf, b2 = tinyf;
    int c = 0;
    for (int w = 0; w < nwarp; ++w) {
      top2f(b1, b2, w1[w], w2[w]);
      c += wc[w];
    }
    d.part[2 * blockIdx.x] = __float_as_uint(b1);
    d.part[2 * blockIdx.x + 1] = __float_as_uint(b2);
    if (!second) {
      d.part1[2 * blockIdx.x] = __float_as_uint(b1);
      d.part1[2 * blockIdx.x + 1] = __float_as_uint(b2);
    }
    if (p.rho_fused) {
      // a clean block of the second call: the first call's count
      if (second && (int)blockIdx.x * kSpan < n_slots && d.dirty[blockIdx.x] == 0)
        c = d.part_cnt[2 * blockIdx.x];
      if (!second) d.part_cnt[2 * blockIdx.x] = c;
      d.part_cnt[2 * blockIdx.x + 1] = c;
    }
    __threadfence();
    unsigned t = atomicAdd(&sc->ticket, 1u);
    last = (t == (unsigned)nu - 1u);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  // last block of this replica: FP32 top-2 over the replica's partials
  float b1 = tinyf, b2 = tinyf;
  for (int b = b0 + threadIdx.x; b < b0 + nu; b += blockDim.x)
    top2f(b1, b2, __uint_as_float((unsigned)__ldcg(d.part + 2 * b)),
          __uint_as_float((unsigned)__ldcg(d.part + 2 * b + 1)));
  for (int off = 16; off > 0; off >>= 1) {
    float c1 = __shfl_down_sync(0xffffffffu, b1, off);
    float c2 = __shfl_down_sync(0xffffffffu, b2, off);
    top2f(b1, b2, c1, c2);
  }
  __syncthreads();
  if (lane == 0) {
    w1[wid] = b1;
    w2[wid] = b2;
  }
  __syncthreads();
  if (p.rho_fused && second) {  // calc_rho (dana.F90:521-549) of the replica
    __shared__ int s_c;
    if (threadIdx.x == 0) s_c = 0;
    __syncthreads();
    int c = 0;
    for (int b = b0 + threadIdx.x; b < b0 + nu; b += blockDim.x)
      c += __ldcg(d.part_cnt + 2 * b + 1);
    if (c) atomicAdd(&s_c, c);
    __syncthreads();
    if (threadIdx.x == 0) {
      const double vol = R.box[0] * R.box[1] * (czt - cz0);
      sc->rho = (double)s_c / vol;
    }
  }
  __shared__ int s_dec;
  __shared__ float s_thr;
  if (threadIdx.x == 0) {
    float F1 = tinyf, F2 = tinyf;
    for (int w = 0; w < nwarp; ++w) top2f(F1, F2, w1[w], w2[w]);
    float sum = sqrtf(F1) + sqrtf(F2);
    int dec;  // 0 keep, 1 rebuild, 2 undecided: dispmax_exact_kernel decides
    if (!sc->listed) dec = 1;
    else if (sum + 4.0f * e < (float)p.skin) dec = 0;
    else if (sum - 4.0f * e > (float)p.skin) dec = 1;
    else dec = 2;
    sc->dec = dec;
    sc->thr = sqrtf(F2) - 3.0f * e;
    sc->dt_tests += 1;
    if (dec == 2) sc->dt_exact += 1;
    sc->ticket = 0;
    if (dec != 2) decide_rebuild(d, sc, dec);
    s_dec = dec;
    s_thr = sc->thr;
  }
  __syncthreads();
  if (s_dec != 2) return;
  // Undecided: the exact pass walks the spans in use whose FP32 maximum
  // reaches the threshold (an atom's rdf is at most its span's maximum, and
  // sqrtf is correctly rounded, hence monotone), listed here contiguously.
  int nsp = 0;
  for (int b = threadIdx.x; b < nu; b += blockDim.x)
    nsp += sqrtf(__uint_as_float((unsigned)__ldcg(d.part + 2 * (b0 + b)))) >= s_thr;
  int tot;
  const int pre = blk_scan_excl(nsp, &tot);
  __shared__ int s_beg;
  if (threadIdx.x == 0) {
    s_beg = tot ? atomicAdd(&d.g->n_xspan, tot) : 0;
    sc->xbeg = s_beg;
    sc->xcnt = tot;
  }
  __syncthreads();
  int at = s_beg + pre;
  for (int b = threadIdx.x; b < nu; b += blockDim.x)
    if (sqrtf(__uint_as_float((unsigned)__ldcg(d.part + 2 * (b0 + b)))) >= s_thr)
      d.xspan[at++] = b0 + b;
}

// The replicas whose FP32 top-2 lies within the margins of the skin: the
// exact FP64 top-2 over the candidates (sqrt(rdf) >= sqrt(F2) - 3e, which
// holds for every atom of the exact top-2), on a fixed grid.  First the spans
// pbc_dispmax listed (one block per span in turn; the last span of a replica
// merges its partials and decides), then each block counts the replicas of
// its share that were decided without the pass.  The replica count that
// reaches nrep makes its block the last: it prefixes the rows of the replicas
// that rebuild (the list build walks only those) and opens the rebuild
// subgraph if any.  With no replica undecided the launch is one short wave.
constexpr int kExactGrid = 152 * 4;
__global__ void __launch_bounds__(kBlock) dispmax_exact_kernel(
    Dev d, KParams p, int cond, cudaGraphConditionalHandle cond_handle) {
  DML_GRID_WAIT();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nwarp = blockDim.x >> 5;
  const unsigned long long tiny = (unsigned long long)__double_as_longlong(1.e-16);
  __shared__ unsigned long long x1[32], x2[32];
  __shared__ int s_close, s_lastrep;
  __shared__ int s_cnt;
  if (threadIdx.x == 0) {
    s_lastrep = 0;
    s_cnt = 0;
  }
  const int nx = d.g->n_xspan;
  for (int t = blockIdx.x; t < nx; t += gridDim.x) {
    const int sp = d.xspan[t];
    const int rep = d.rep_of[sp * kSpan];
    const RepConst& R = d.rc[rep];
    Scalars* sc = d.sc + rep;
    const int n_slots = R.base + sc->n_slots;
    const float thr = sc->thr;
    unsigned long long e1 = tiny, e2 = tiny;
#pragma unroll
    for (int u = 0; u < kSlotU; ++u) {
      const int q = sp * kSpan + u * kBlock + (int)threadIdx.x;
      if (q < n_slots && d.state[q] == ST_LIVE) {
        const float rdf = disp2f(d.posf[q], d.posf_old[q]);
        if (rdf == rdf && sqrtf(rdf) >= thr) {
          const double4 P = d.pos[q], O = d.pos_old[q];
          const double rd = dot3(P.x - O.x, P.y - O.y, P.z - O.z);
          if (rd == rd) top2_merge(e1, e2, (unsigned long long)__double_as_longlong(rd), tiny);
        }
      }
    }
    for (int off = 16; off > 0; off >>= 1) {
      unsigned long long c1 = __shfl_down_sync(0xffffffffu, e1, off);
      unsigned long long c2 = __shfl_down_sync(0xffffffffu, e2, off);
      top2_merge(e1, e2, c1, c2);
    }
    if (lane == 0) {
      x1[wid] = e1;
      x2[wid] = e2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned long long f1 = tiny, f2 = tiny;
      for (int w = 0; w < nwarp; ++w) top2_merge(f1, f2, x1[w], x2[w]);
      d.xpart[2 * t] = f1;
      d.xpart[2 * t + 1] = f2;
      __threadfence();
      const unsigned tk = atomicAdd(&sc->ticket, 1u);
      s_close = tk == (unsigned)sc->xcnt - 1u;
    }
    __syncthreads();
    if (s_close) {
      // the replica's last listed span: its partials merged, the decision
      __threadfence();
      unsigned long long f1 = tiny, f2 = tiny;
      const int xb = sc->xbeg, xc = sc->xcnt;
      for (int b = xb + threadIdx.x; b < xb + xc; b += blockDim.x)
        top2_merge(f1, f2, __ldcg(d.xpart + 2 * b), __ldcg(d.xpart + 2 * b + 1));
      for (int off = 16; off > 0; off >>= 1) {
        unsigned long long c1 = __shfl_down_sync(0xffffffffu, f1, off);
        unsigned long long c2 = __shfl_down_sync(0xffffffffu, f2, off);
        top2_merge(f1, f2, c1, c2);
      }
      __syncthreads();
      if (lane == 0) {
        x1[wid] = f1;
        x2[wid] = f2;
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        unsigned long long g1 = tiny, g2 = tiny;
        for (int w = 0; w < nwarp; ++w) top2_merge(g1, g2, x1[w], x2[w]);
        const double d1 = __longlong_as_double((long long)g1);
        const double d2 = __longlong_as_double((long long)g2);
        decide_rebuild(d, sc, sqrt(d1) + sqrt(d2) > p.skin ? 1 : 0);
        sc->ticket = 0;
        s_cnt += 1;
      }
    }
    __syncthreads();
  }
  // the replicas of this block's share decided without the exact pass (an
  // undecided replica with no listed span has no candidate: its exact top-2
  // is empty)
  int cnt = 0;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < d.nrep; r += gridDim.x * blockDim.x) {
    Scalars* sc = d.sc + r;
    if (sc->dec != 2) {
      ++cnt;
    } else if (sc->xcnt == 0) {
      const double t1 = __longlong_as_double((long long)tiny);
      decide_rebuild(d, sc, sqrt(t1) + sqrt(t1) > p.skin ? 1 : 0);
      ++cnt;
    }
  }
  for (int off = 16; off > 0; off >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, off);
  __syncthreads();
  if (lane == 0 && cnt) atomicAdd(&s_cnt, cnt);
  __syncthreads();
  if (threadIdx.x == 0 && s_cnt) {
    __threadfence();
    const unsigned t2 = atomicAdd(&d.g->ticket_rep, (unsigned)s_cnt);
    s_lastrep = t2 + (unsigned)s_cnt == (unsigned)d.nrep;
  }
  __syncthreads();
  if (!s_lastrep) return;
  // The last replica to decide: the rows of the replicas that rebuild (the
  // list build walks only those) and their cell chunks (the cell sort walks
  // only those), then the rebuild subgraph opens if any.
  __threadfence();
  __shared__ int carry, carry2;
  if (threadIdx.x == 0) {
    carry = 0;
    carry2 = 0;
  }
  __syncthreads();
  for (int base0 = 0; base0 < d.nrep; base0 += blockDim.x) {
    const int r = base0 + threadIdx.x;
    int v = 0, v2 = 0;
    if (r < d.nrep) {
      const volatile Scalars* q = d.sc + r;
      const RepConst& Rr = d.rc[r];
      v = q->rebuild ? q->n_rank : 0;
      v2 = q->rebuild && Rr.use_cells ? (Rr.ncell + kCellChunk - 1) / kCellChunk : 0;
    }
    int x = v, x2 = v2;
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, x, o), y2 = __shfl_up_sync(0xffffffffu, x2, o);
      if (lane >= o) {
        x += y;
        x2 += y2;
      }
    }
    __shared__ int wsum[32], wsum2[32];
    if (lane == 31) {
      wsum[wid] = x;
      wsum2[wid] = x2;
    }
    __syncthreads();
    if (wid == 0) {
      int w = lane < nwarp ? wsum[lane] : 0, w2 = lane < nwarp ? wsum2[lane] : 0;
      for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, w, o), y2 = __shfl_up_sync(0xffffffffu, w2, o);
        if (lane >= o) {
          w += y;
          w2 += y2;
        }
      }
      wsum[lane] = w;
      wsum2[lane] = w2;
    }
    __syncthreads();
    const int pre = (wid > 0 ? wsum[wid - 1] : 0) + x - v;
    const int pre2 = (wid > 0 ? wsum2[wid - 1] : 0) + x2 - v2;
    if (r < d.nrep) {
      d.reb_pre[r] = carry + pre;
      d.rebc_pre[r] = carry2 + pre2;
    }
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) {
      carry += pre + v;
      carry2 += pre2 + v2;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    d.reb_pre[d.nrep] = carry;
    d.rebc_pre[d.nrep] = carry2;
    int any = atomicAdd(&d.g->any_rebuild, 0);
    d.g->ticket_rep = 0;
    d.g->n_xspan = 0;  // every listed span has been walked
    if (any) d.g->near_stale = 1;  // lists change: the near entries too
    if (cond) cudaGraphSetConditional(cond_handle, any ? 1u : 0u);
  }
}

// update() (Neighbor.F90:608-633) part 1: pos_old = pos, limbo cleaned
// (igroup_clean, Groups.F90:1036-1053), cell index of every hs%b slot
// (cgroup_sort_atom, Cells.F90:281-302) and the per-cell counts.
__device__ __forceinline__ void rebuild_prep_at(Dev d, KParams p, int n_slots, int n_b, int cells_only, int rep, int pos) {
  const RepConst& R = d.rc[rep];
  Scalars* sc = d.sc + rep;
  n_slots = R.base + sc->n_slots;
  n_b = R.base + sc->n_b;
  if (blockIdx.x == 0 && threadIdx.x == 0) d.g->n_big = 0;  // cell_order's list
  if (!cells_only && !sc->rebuild) return;
  const int s = pos;
  if (!cells_only && s == R.base) sc->nlimbo = 0;
  if (!cells_only && s < n_slots) {
    int st = d.state[s];
    if (st == ST_LIVE) {
      d.pos_old[s] = d.pos[s];
      d.posf_old[s] = d.posf[s];
    } else if (st == ST_LIMBO) {
      d.state[s] = ST_NULL;
      atomicMin(&sc->free_lo, s - R.base);  // the slot is free again
    }
  }
  if (R.use_cells && s < n_b) {
    int hs = d.b2hs[s];
    if (hs < 0) {
      d.cell_of[s] = -1;
      return;
    }
    int c1, c2, c3;
    cell_index3(R, d.posf[hs], d.pos + hs, c1, c2, c3);
    if (c1 < 0 || c2 < 0 || c3 < 0 || c1 > R.ncells[0] + 1 || c2 > R.ncells[1] + 1 ||
        c3 > R.ncells[2] + 1) {
      raise_error(d.g, DML_E_OUT_OF_TESSELLATION, hs);
      d.cell_of[s] = -1;
      return;
    }
    // the 27-cell stencil never visits the halo: searches over cells that
    // must see every atom (GCMC) fall back to full scans for this replica
    if (c1 == 0 || c2 == 0 || c3 == 0 || c1 > R.ncells[0] || c2 > R.ncells[1] ||
        c3 > R.ncells[2])
      sc->halo = 1;
    // the sort for gcmc_run holds only the atoms its searches can reach
    if (cells_only && !R.gl_all && !((R.gl_cmask >> c3) & 1ull)) {
      d.cell_of[s] = -1;
      return;
    }
    int lin = R.cell_off + (c3 * R.head_dim[1] + c2) * R.head_dim[0] + c1;
    d.cell_of[s] = lin;
    atomicAdd(&d.cell_count[lin], 1);
  }
}

__global__ void rebuild_prep_kernel(Dev d, KParams p, int n_slots, int n_b, int cells_only) {
  DML_GRID_WAIT();
  const int rep = block_rep(d);
#pragma unroll
  for (int u = 0; u < kSlotU; ++u) rebuild_prep_at(d, p, n_slots, n_b, cells_only, rep, span_pos(u));
}

// Exclusive scan of one replica's cell counts over the cells [c0, c1) of the
// replica (one block), continuing from *carry; cell c1 receives the end.
__device__ void cell_scan_range(const Dev& d, const RepConst& R, int c0, int c1, int* carry) {
  __shared__ int wsum[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int base = c0; base < c1; base += blockDim.x) {
    const int i = base + threadIdx.x;
    const int v = i < c1 ? d.cell_count[R.cell_off + i] : 0;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[wid] = x;
    __syncthreads();
    if (wid == 0) {
      int ws = lane < (int)(blockDim.x >> 5) ? wsum[lane] : 0;
      for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, ws, o);
        if (lane >= o) ws += y;
      }
      wsum[lane] = ws;
    }
    __syncthreads();
    const int pre = (wid > 0 ? wsum[wid - 1] : 0) + x - v;
    if (i < c1) {
      d.cell_start[R.cell_off + i] = *carry + pre;
      d.cell_fill[R.cell_off + i] = 0;
    }
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) *carry += pre + v;
    __syncthreads();
  }
  if (threadIdx.x == 0) d.cell_start[R.cell_off + c1] = *carry;
  __syncthreads();
}

// The cell sort of gcmc_run on the device-wide cell arrays runs for the
// replicas whose trials run sequentially (gcmc_kernel): their sorts only.
__device__ __forceinline__ bool gcmc_sorts(const Dev& d, int rep, int par) {
  return !par || !d.grp[rep].fast;
}

// The cell starts of one replica (one block per replica), from its first
// position: its cell_atoms range is [base, base + cap).  A full sort covers
// every cell and the sentinel after the last; the sort for gcmc_run covers
// the runs of z layers its searches reach, each followed by its end.
__global__ void cell_scan_kernel(Dev d, int force, int par) {
  DML_GRID_WAIT();
  const RepConst& R = d.rc[blockIdx.x];
  const Scalars* sc = d.sc + blockIdx.x;
  if (!R.use_cells) return;
  if (!force && !sc->rebuild) return;
  if (force && !gcmc_sorts(d, blockIdx.x, par)) return;
  __shared__ int carry;
  if (threadIdx.x == 0) carry = R.base;
  __syncthreads();
  if (!force || R.gl_all) {
    cell_scan_range(d, R, 0, R.ncell, &carry);  // cell ncell is the sentinel
    return;
  }
  const int layer = R.head_dim[0] * R.head_dim[1];
  for (int a = 1; a <= R.ncells[2]; ++a) {
    if (!((R.gl_mask >> a) & 1ull)) continue;
    int b = a;
    while (b + 1 <= R.ncells[2] && ((R.gl_mask >> (b + 1)) & 1ull)) ++b;
    cell_scan_range(d, R, a * layer, (b + 1) * layer, &carry);
    a = b;
  }
}

__device__ __forceinline__ void cell_scatter_at(Dev d, int n_b, int force, int rep, int pos) {
  const RepConst& R = d.rc[rep];
  Scalars* sc = d.sc + rep;
  n_b = R.base + sc->n_b;
  if (!R.use_cells) return;            // no cells: cell_of is never written
  if (!force && !sc->rebuild) return;  // its cell_of entries are from an older sort
  const int b = pos;
  if (b >= n_b) return;
  int c = d.cell_of[b];
  if (c < 0) return;
  int idx = d.cell_start[c] + atomicAdd(&d.cell_fill[c], 1);
  d.cell_atoms[idx] = b;
}

__global__ void cell_scatter_kernel(Dev d, int n_b, int force) {
  DML_GRID_WAIT();
  const int rep = block_rep(d);
#pragma unroll
  for (int u = 0; u < kSlotU; ++u) cell_scatter_at(d, n_b, force, rep, span_pos(u));
}

// Orders each cell by descending hs%b slot: the chain order of
// cgroup_sort (Cells.F90:267-302), which prepends slots in increasing order.
// One warp per cell; the sorted cell goes to comp_members (scratch) and is
// copied back as hs slots (what the list stores).
__device__ __forceinline__ void cell_order_cell(const Dev& d, int c) {
  int lane = threadIdx.x & 31;
  // counted in this sort (replicas that do not sort keep zero counts)
  int num = __shfl_sync(0xffffffffu, lane == 0 ? d.cell_count[c] : 0, 0);
  if (num == 0) return;
  int start = d.cell_start[c];
  if (lane == 0) d.cell_count[c] = 0;
  if (num == 1 && lane == 0) d.cell_atoms[start] = d.b2hs[d.cell_atoms[start]];
  if (num <= 1) return;
  const int* seg = d.cell_atoms + start;
  int* tmp = d.comp_members + start;  // scratch of n_b entries
  for (int i = lane; i < num; i += 32) {
    int v = seg[i];
    int rnk = 0;
    for (int q = 0; q < num; ++q) rnk += seg[q] > v;
    tmp[rnk] = v;
  }
  __syncwarp();
  for (int i = lane; i < num; i += 32) ((int*)seg)[i] = d.b2hs[tmp[i]];
}

// Cells of at most kSmallCell atoms are ordered by one thread each (a
// sorting network in registers); larger ones are listed for a warp each.
// A block covers one chunk of kCellChunk cells of one replica; chunks of
// replicas that do not sort (and, for gcmc_run's sort, of z layers its
// searches do not reach) are skipped whole.
constexpr int kSmallCell = 16;
__device__ void cell_order_chunk(const Dev& d, const RepConst& R, int force, int chunk) {
  const int c0 = chunk * kCellChunk;
  if (force && !R.gl_all) {
    const int layer = R.head_dim[0] * R.head_dim[1];
    const int l0 = c0 / layer, l1 = (min(c0 + kCellChunk, R.ncell) - 1) / layer;
    const unsigned long long span =
        (l1 - l0 >= 63 ? ~0ull : ((2ull << (l1 - l0)) - 1ull)) << l0;
    if (l0 > 63 || !(R.gl_mask & span)) return;
  }
  // The thread's four cells: counts and starts loaded together, then the
  // one-atom cells (most occupied ones, nothing to order) in two batched
  // rounds (the atom, its hs slot); the others one by one below.
  constexpr int U = kCellChunk / kBlock;
  int nums[U], sts[U], one[U];
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int ci = c0 + u * kBlock + (int)threadIdx.x;
    nums[u] = ci < R.ncell ? d.cell_count[R.cell_off + ci] : 0;
    sts[u] = ci < R.ncell ? d.cell_start[R.cell_off + ci] : 0;
  }
#pragma unroll
  for (int u = 0; u < U; ++u) one[u] = nums[u] == 1 ? d.cell_atoms[sts[u]] : -1;
#pragma unroll
  for (int u = 0; u < U; ++u)
    if (nums[u] == 1) {
      d.cell_count[R.cell_off + c0 + u * kBlock + (int)threadIdx.x] = 0;
      d.cell_atoms[sts[u]] = d.b2hs[one[u]];
    }
#pragma unroll 1
  for (int u = 0; u < U; ++u) {
    const int num = nums[u];
    if (num <= 1) continue;
    const int c = R.cell_off + c0 + u * kBlock + (int)threadIdx.x;
    if (num > kSmallCell) {
      d.big_cells[atomicAdd(&d.g->n_big, 1)] = c;
      continue;
    }
    d.cell_count[c] = 0;
    const int start = sts[u];
    if (num == 2) {
      const int a = d.cell_atoms[start], b = d.cell_atoms[start + 1];
      d.cell_atoms[start] = d.b2hs[max(a, b)];
      d.cell_atoms[start + 1] = d.b2hs[min(a, b)];
      continue;
    }
    int v[kSmallCell];
#pragma unroll
    for (int k = 0; k < kSmallCell; ++k) v[k] = k < num ? d.cell_atoms[start + k] : -1;
    // descending odd-even transposition sort (the b slots are distinct, >= 0)
#pragma unroll
    for (int rnd = 0; rnd < kSmallCell; ++rnd) {
#pragma unroll
      for (int k = rnd & 1; k + 1 < kSmallCell; k += 2) {
        int a = v[k], b = v[k + 1];
        v[k] = max(a, b);
        v[k + 1] = min(a, b);
      }
    }
#pragma unroll
    for (int k = 0; k < kSmallCell; ++k)
      if (k < num) d.cell_atoms[start + k] = d.b2hs[v[k]];
  }
}

__global__ void cell_order_small_kernel(Dev d, int force, int par) {
  DML_GRID_WAIT();
  if (!force && !d.g->any_rebuild) return;
  const int rep = d.cch_rep[blockIdx.x];
  const RepConst& R = d.rc[rep];
  if (!R.use_cells) return;
  if (!force && !d.sc[rep].rebuild) return;
  if (force && !gcmc_sorts(d, rep, par)) return;
  cell_order_chunk(d, R, force, blockIdx.x - R.cch0);
}

__device__ int blk_scan_excl(int v, int* total) {
  // exclusive scan over a block of up to 1024 threads
  __shared__ int ws[32];
  __shared__ int tot;
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int nw = (blockDim.x + 31) >> 5;
    int w = lane < nw ? ws[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    ws[lane] = w;
    if (lane == 31) tot = w;
  }
  __syncthreads();
  int r = (wid > 0 ? ws[wid - 1] : 0) + x - v;
  *total = tot;
  __syncthreads();
  return r;
}

// The list rebuild's cell sort over the chunks of the replicas that rebuild
// only (rebc_pre), on a fixed grid: a chunk's replica and index within it.
__device__ __forceinline__ void reb_chunk(const Dev& d, int g, int& rep, int& q) {
  int lo = 0, hi = d.nrep - 1;  // last replica whose prefix is <= g
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (d.rebc_pre[mid] <= g) lo = mid; else hi = mid - 1;
  }
  rep = lo;
  q = g - d.rebc_pre[lo];
}

// Cell starts in three passes: the count of every chunk, the prefix over a
// replica's chunks (from its first cell_atoms place, with the sentinel
// cell's start), and each chunk's own prefix.
__global__ void cell_chunk_sum_kernel(Dev d) {
  DML_GRID_WAIT();
  __shared__ int ws[kBlock / 32];
  const int total = d.rebc_pre[d.nrep];
  for (int g = blockIdx.x; g < total; g += gridDim.x) {
    int rep, q;
    reb_chunk(d, g, rep, q);
    const RepConst& R = d.rc[rep];
    int v = 0;
#pragma unroll
    for (int u = 0; u < kCellChunk / kBlock; ++u) {
      const int ci = q * kCellChunk + u * kBlock + (int)threadIdx.x;
      if (ci < R.ncell) v += d.cell_count[R.cell_off + ci];
    }
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
      int t = 0;
      for (int w = 0; w < kBlock / 32; ++w) t += ws[w];
      d.chunk_sum[R.cch0 + q] = t;
    }
    __syncthreads();
  }
}

__global__ void cell_chunk_scan_kernel(Dev d) {
  DML_GRID_WAIT();
  const int rep = blockIdx.x;
  const RepConst& R = d.rc[rep];
  if (!R.use_cells || !d.sc[rep].rebuild) return;
  const int nq = (R.ncell + kCellChunk - 1) / kCellChunk;
  __shared__ int carry;
  if (threadIdx.x == 0) carry = R.base;
  __syncthreads();
  for (int q0 = 0; q0 < nq; q0 += blockDim.x) {
    const int q = q0 + (int)threadIdx.x;
    const int v = q < nq ? d.chunk_sum[R.cch0 + q] : 0;
    int tot;
    const int pre = blk_scan_excl(v, &tot);
    if (q < nq) d.chunk_base[R.cch0 + q] = carry + pre;
    __syncthreads();
    if (threadIdx.x == 0) carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) d.cell_start[R.cell_off + R.ncell] = carry;  // the sentinel cell
}

__global__ void cell_chunk_fill_kernel(Dev d) {
  DML_GRID_WAIT();
  const int total = d.rebc_pre[d.nrep];
  for (int g = blockIdx.x; g < total; g += gridDim.x) {
    int rep, q;
    reb_chunk(d, g, rep, q);
    const RepConst& R = d.rc[rep];
    int v[kCellChunk / kBlock], s = 0;
#pragma unroll
    for (int u = 0; u < kCellChunk / kBlock; ++u) {  // 4 consecutive cells per thread
      const int ci = q * kCellChunk + (int)threadIdx.x * (kCellChunk / kBlock) + u;
      v[u] = ci < R.ncell ? d.cell_count[R.cell_off + ci] : 0;
      s += v[u];
    }
    int tot;
    int run = d.chunk_base[R.cch0 + q] + blk_scan_excl(s, &tot);
#pragma unroll
    for (int u = 0; u < kCellChunk / kBlock; ++u) {
      const int ci = q * kCellChunk + (int)threadIdx.x * (kCellChunk / kBlock) + u;
      if (ci < R.ncell) {
        d.cell_start[R.cell_off + ci] = run;
        d.cell_fill[R.cell_off + ci] = 0;
      }
      run += v[u];
    }
  }
}

// The rebuild's in-cell order over the same chunks.
__global__ void cell_order_reb_kernel(Dev d) {
  DML_GRID_WAIT();
  const int total = d.rebc_pre[d.nrep];
  for (int g = blockIdx.x; g < total; g += gridDim.x) {
    int rep, q;
    reb_chunk(d, g, rep, q);
    cell_order_chunk(d, d.rc[rep], 0, q);
    __syncthreads();
  }
}

// gcmc_run's sort with the parallel trials: one block per replica, which
// leaves at once unless the replica's trials run sequentially (the rare
// case, where its chunks are ordered one after another).
__global__ void gcmc_order_kernel(Dev d) {
  DML_GRID_WAIT();
  const int rep = blockIdx.x;
  const RepConst& R = d.rc[rep];
  if (!R.use_cells || !gcmc_sorts(d, rep, 1)) return;
  for (int q = 0; q < (R.ncell + kCellChunk - 1) / kCellChunk; ++q) cell_order_chunk(d, R, 1, q);
}

__global__ void cell_order_big_kernel(Dev d, int force) {
  DML_GRID_WAIT();
  if (!force && !d.g->any_rebuild) return;
  const int nw = gridDim.x * (blockDim.x >> 5);
  const int nb = d.g->n_big;
  for (int q = warp_id_global(); q < nb; q += nw) cell_order_cell(d, d.big_cells[q]);
}

// ngroup_cells (Neighbor.F90:465-548): one warp per hs%ref member, the 27
// stencil cells in map order (Cells.F90:28-36), each cell in chain order,
// wrapped as cell_pbc with mic (Cells.F90:378-404), `rd < (rc+skin)^2`.
__device__ __forceinline__ void list_cells_row(const Dev& d, const KParams& p, int r,
                                               int* tab) {
  int lane = threadIdx.x & 31;
  const int rep = d.rep_of[r];
  const RepConst& R = d.rc[rep];
  Scalars* sc = d.sc + rep;
  if (!sc->rebuild || !R.use_cells || R.list_thread) return;
  if (r - R.base >= sc->n_rank) return;
  int h = d.ref[r];
  if (h < 0) return;
  double4 P = d.pos[h];
  float4 Pf = d.posf[h];
  int rc[3];
  cell_index3(R, Pf, d.pos + h, rc[0], rc[1], rc[2]);
  if (rc[0] == INT_MIN || rc[1] == INT_MIN || rc[2] == INT_MIN) {
    if (lane == 0) raise_error(d.g, DML_E_OUT_OF_TESSELLATION, h);
    return;
  }
  // Lane q < 27 takes stencil cell q (map order): its start in tab[q], the
  // exclusive prefix of the cell sizes in tab[27 + q], the total in tab[54].
  // The 27 cells then form one index space f that keeps the list order
  // (cell by cell, each cell in chain order), scanned 32 entries at a time.
  __syncwarp();
  int num = 0;
  bool bad = false;
  if (lane < 27) {
    int nc[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      int t = map_off(lane, k) + rc[k] - 1;
      t = (t + R.ncells[k]) % R.ncells[k];
      nc[k] = t + 1;
      if (nc[k] < 0 || nc[k] > R.ncells[k] + 1) bad = true;
    }
    if (!bad) {
      int c = R.cell_off + (nc[2] * R.head_dim[1] + nc[1]) * R.head_dim[0] + nc[0];
      int st = d.cell_start[c];
      num = d.cell_start[c + 1] - st;
      tab[lane] = st;
    }
  }
  if (__any_sync(0xffffffffu, bad)) {
    if (lane == 0) raise_error(d.g, DML_E_OUT_OF_TESSELLATION, h);
    return;
  }
  int x = num;
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane < 27) tab[27 + lane] = x - num;
  const int T = __shfl_sync(0xffffffffu, x, 26);
  __syncwarp();
  int* row = d.list + (size_t)h * p.mnb;
  int cnt = 0;
  for (int base = 0; base < T; base += 32) {
    const int f = base + lane;
    bool inc = false;
    int j = -1;
    if (f < T) {
      int lo = 0, hi = 26;  // the cell holding f: largest q with prefix <= f
      while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (tab[27 + mid] <= f) lo = mid; else hi = mid - 1;
      }
      j = d.cell_atoms[tab[lo] + f - tab[27 + lo]];  // hs slot
      if (j != h) {
        float4 Q = d.posf[j];
        float fx, fy, fz;
        vdist_nint_f(R, Q, Pf, fx, fy, fz);
        float drf = fx * fx + fy * fy + fz * fz;
        if (drf < R.rlist_lo2) {
          inc = true;
        } else if (drf <= R.rlist_hi2) {
          double vx, vy, vz;
          vdist_nint(R, d.pos[j], P, vx, vy, vz);
          double rd = dot3(vx, vy, vz);
          inc = rd < p.rlist2;
        }
      }
    }
    unsigned bal = __ballot_sync(0xffffffffu, inc);
    int pre = __popc(bal & ((1u << lane) - 1u));
    if (inc && cnt + pre < p.mnb) row[cnt + pre] = j;
    cnt += __popc(bal);
  }
  if (lane == 0) {
    if (cnt > p.mnb) {
      raise_error(d.g, DML_E_NEIGH_OVERFLOW, h);
      cnt = p.mnb;
    }
    d.nn[h] = cnt;
    atomicMax(&sc->max_nn, cnt);
  }
}

// The same rows, one thread per row, for replicas whose cells hold few
// atoms (RepConst::list_thread): a warp per row there spends most of its
// instructions on the 27-cell set-up of a handful of candidates.  The
// thread walks the 27 stencil cells in map order and each cell in chain
// order, with the warp version's inclusion test, so the rows are the same.
// Returns the row length (or -1 when the thread had no row).
__device__ __forceinline__ int list_cells_row_thread(const Dev& d, const KParams& p, int r,
                                                     int rep) {
  const RepConst& R = d.rc[rep];
  Scalars* sc = d.sc + rep;
  if (!sc->rebuild || !R.use_cells || !R.list_thread) return -1;
  if (r - R.base >= sc->n_rank) return -1;
  const int h = d.ref[r];
  if (h < 0) return -1;
  const double4 P = d.pos[h];
  const float4 Pf = d.posf[h];
  int rc[3];
  cell_index3(R, Pf, d.pos + h, rc[0], rc[1], rc[2]);
  if (rc[0] == INT_MIN || rc[1] == INT_MIN || rc[2] == INT_MIN) {
    raise_error(d.g, DML_E_OUT_OF_TESSELLATION, h);
    return -1;
  }
  // the wrapped cell coordinate of offsets -1, 0, +1 along each axis
  // (cell_pbc), held in registers and selected per stencil cell
  int wm[3], w0[3], wp[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    wm[k] = (rc[k] - 2 + R.ncells[k]) % R.ncells[k] + 1;
    w0[k] = (rc[k] - 1 + R.ncells[k]) % R.ncells[k] + 1;
    wp[k] = (rc[k] + R.ncells[k]) % R.ncells[k] + 1;
    if (min(wm[k], min(w0[k], wp[k])) < 0 || max(wm[k], max(w0[k], wp[k])) > R.ncells[k] + 1) {
      raise_error(d.g, DML_E_OUT_OF_TESSELLATION, h);
      return -1;
    }
  }
  int* row = d.list + (size_t)h * p.mnb;
  int cnt = 0;
  // The bounds of all 27 stencil cells first, their loads issued together
  // (a bit per non-empty cell), then the non-empty cells in map order: most
  // cells of a sparse replica are empty, and walking them one by one put a
  // load latency per cell on the row's chain.
  auto stencil_cell = [&](int q) {
    int nc[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int o = map_off(q, k);
      nc[k] = o < 0 ? wm[k] : (o == 0 ? w0[k] : wp[k]);
    }
    return R.cell_off + (nc[2] * R.head_dim[1] + nc[1]) * R.head_dim[0] + nc[0];
  };
  unsigned ne = 0u;
#pragma unroll
  for (int q = 0; q < 27; ++q) {
    const int c = stencil_cell(q);
    if (d.cell_start[c + 1] > d.cell_start[c]) ne |= 1u << q;
  }
  // The candidates of the non-empty cells (map order, chain order within a
  // cell) as one stream: while candidate k is tested, the FP32 position of
  // k + 1 and the hs slot of k + 2 are loaded, so that the stream waits on
  // one load latency per candidate instead of two.
  int fi = 0, fe = 0;  // the next stream position to fetch: cell_atoms[fi], fi < fe
  auto fetch = [&]() -> int {
    if (fi >= fe) {
      if (ne == 0u) return -1;
      const int c = stencil_cell(__ffs(ne) - 1);
      ne &= ne - 1u;
      fi = d.cell_start[c];
      fe = d.cell_start[c + 1];
    }
    return d.cell_atoms[fi++];  // hs slot
  };
  int j1 = fetch();
  int j2 = j1 >= 0 ? fetch() : -1;
  float4 Q1 = j1 >= 0 ? d.posf[j1] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 1
  while (j1 >= 0) {
    const int j3 = j2 >= 0 ? fetch() : -1;
    const float4 Q2 = j2 >= 0 ? d.posf[j2] : make_float4(0.f, 0.f, 0.f, 0.f);
    if (j1 != h) {
      float fx, fy, fz;
      vdist_nint_f(R, Q1, Pf, fx, fy, fz);
      const float drf = fx * fx + fy * fy + fz * fz;
      bool inc = false;
      if (drf < R.rlist_lo2) {
        inc = true;
      } else if (drf <= R.rlist_hi2) {
        double vx, vy, vz;
        vdist_nint(R, d.pos[j1], P, vx, vy, vz);
        inc = dot3(vx, vy, vz) < p.rlist2;
      }
      if (inc) {
        if (cnt < p.mnb) row[cnt] = j1;
        ++cnt;
      }
    }
    j1 = j2;
    Q1 = Q2;
    j2 = j3;
  }
  if (cnt > p.mnb) {
    raise_error(d.g, DML_E_NEIGH_OVERFLOW, h);
    cnt = p.mnb;
  }
  d.nn[h] = cnt;
  return cnt;
}

__global__ void __launch_bounds__(256, 5) list_cells_thread_kernel(Dev d, KParams p) {
  DML_GRID_WAIT();
  const int total = d.reb_pre[d.nrep];  // rows of the replicas that rebuild
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    const int r = row_rank_in(d, d.reb_pre, i);
    const int rep = d.rep_of[r];
    const int cnt = list_cells_row_thread(d, p, r, rep);
    // the longest row per replica: one atomic per replica present in the warp
    const unsigned act = __activemask();
    const unsigned grp = __match_any_sync(act, rep);
    const int m = __reduce_max_sync(grp, cnt > 0 ? cnt : 0);
    if ((int)(threadIdx.x & 31) == __ffs(grp) - 1 && m > 0) atomicMax(&d.sc[rep].max_nn, m);
  }
}

__global__ void __launch_bounds__(256) list_cells_kernel(Dev d, KParams p, int n_rank) {
  DML_GRID_WAIT();
  __shared__ int tab[8][56];  // per warp: the stencil cells' starts and prefixes
  const int nw = gridDim.x * (blockDim.x >> 5);
  const int total = d.reb_pre[d.nrep];  // rows of the replicas that rebuild
  for (int i = warp_id_global(); i < total; i += nw)
    list_cells_row(d, p, row_rank_in(d, d.reb_pre, i), tab[threadIdx.x >> 5]);
}

// ngroup_verlet (Neighbor.F90:358-424): all hs%b slots in index order,
// `rd > (rc+skin)^2` rejected (so equality is kept), vdistance(ai, aj).
__device__ __forceinline__ void list_verlet_row(const Dev& d, const KParams& p, int r, int n_b) {
  int lane = threadIdx.x & 31;
  const int rep = d.rep_of[r];
  const RepConst& R = d.rc[rep];
  Scalars* sc = d.sc + rep;
  if (!sc->rebuild || R.use_cells) return;
  if (r - R.base >= sc->n_rank) return;
  n_b = R.base + sc->n_b;
  int h = d.ref[r];
  if (h < 0) return;
  double4 P = d.pos[h];
  float4 Pf = d.posf[h];
  int* row = d.list + (size_t)h * p.mnb;
  int cnt = 0;
  for (int base = R.base; base < n_b; base += 32) {
    int b = base + lane;
    bool inc = false;
    int j = -1;
    if (b < n_b) {
      j = d.b2hs[b];
      if (j >= 0 && j != h) {
        float4 Q = d.posf[j];
        float fx, fy, fz;
        vdist_nint_f(R, Pf, Q, fx, fy, fz);
        float drf = fx * fx + fy * fy + fz * fz;
        if (drf < R.rlist_lo2) {
          inc = true;
        } else if (drf <= R.rlist_hi2) {
          double vx, vy, vz;
          vdist_nint(R, P, d.pos[j], vx, vy, vz);
          double rd = dot3(vx, vy, vz);
          inc = !(rd > p.rlist2);
        }
      }
    }
    unsigned bal = __ballot_sync(0xffffffffu, inc);
    int pre = __popc(bal & ((1u << lane) - 1u));
    if (inc && cnt + pre < p.mnb) row[cnt + pre] = j;
    cnt += __popc(bal);
  }
  if (lane == 0) {
    if (cnt > p.mnb) {
      raise_error(d.g, DML_E_NEIGH_OVERFLOW, h);
      cnt = p.mnb;
    }
    d.nn[h] = cnt;
    atomicMax(&sc->max_nn, cnt);
  }
}

__global__ void list_verlet_kernel(Dev d, KParams p, int n_rank, int n_b) {
  DML_GRID_WAIT();
  const int nw = gridDim.x * (blockDim.x >> 5);
  const int total = d.reb_pre[d.nrep];  // rows of the replicas that rebuild
  for (int i = warp_id_global(); i < total; i += nw)
    list_verlet_row(d, p, row_rank_in(d, d.reb_pre, i), n_b);
}

__global__ void rebuild_done_kernel(Dev d) {
  DML_GRID_WAIT();
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r == 0) {
    if (d.g->any_rebuild) d.g->list_builds += 1;
    d.g->any_rebuild = 0;
  }
  if (r >= d.nrep) return;
  if (d.sc[r].rebuild) d.sc[r].listed = 1;
}

// ------------------------------------------------------- overlap_moveback
// The reference resolves hard-core overlaps sequentially in hs%ref order and
// repeats while a pass moved an atom (dana.F90:849-943).  During this phase
// every atom sits either at its integrated position or at old_cg, so any
// pair that can touch during any pass was within rc + 2*delta at the start,
// delta = max |pos - old_cg|.  Atoms linked by such near pairs form
// components; events in different components touch disjoint atoms and
// commute, so each component is replayed in rank order by one thread and
// gives exactly the reference's result.

__global__ void delta_reset_kernel(Global* g) {
  DML_GRID_WAIT();
  g->delta2f_bits = 0u;
}

// Resets the component state and takes delta = max |pos - old_cg| over the
// moving atoms (positions after the integrator; they do not change until
// overlap_moveback except by whole box lengths).
__device__ __forceinline__ void overlap_init_at(Dev d, KParams p, int n_slots, int rep, int pos) {
  const RepConst& R = d.rc[rep];
  Scalars* sc = d.sc + rep;
  n_slots = R.base + sc->n_slots;  // positions in use end here
  const int s = pos;
  if (s == 0) {
    d.g->again = 0;
    d.g->n_comp = 0;
    d.g->comp_total = 0;
    d.g->passes = 1;
  }
  if (s == R.base) {
    sc->passes = 1;
    sc->again2 = 0;
    d.pr_cnt[rep * kCntStride + kCntAct] = 0;
  }
  double dd = 0.0;
  if (s < n_slots) {
    d.uf[s] = s;
    d.active[s] = 0;
    d.comp_size[s] = 0;
    d.comp_fill[s] = 0;
    if (d.state[s] == ST_LIVE && d.rank[s] >= 0) {
      double4 P = d.pos[s], O = d.old_cg[s];
      double x, y, z;
      vdist_nint(R, P, O, x, y, z);
      dd = dot3(x, y, z);
    }
  }
  for (int off = 16; off > 0; off >>= 1) dd = fmax(dd, __shfl_down_sync(0xffffffffu, dd, off));
  if ((threadIdx.x & 31) == 0 && dd > 0.0)
    atomicMax(&d.g->delta2f_bits, __float_as_uint(__double2float_ru(dd)));
}

__global__ void overlap_init_kernel(Dev d, KParams p, int n_slots) {
  DML_GRID_WAIT();
  const int rep = block_rep(d);
#pragma unroll
  for (int u = 0; u < kSlotU; ++u) overlap_init_at(d, p, n_slots, rep, span_pos(u));
}

// Near entries of hs%ref members: list entries within rc + 2 delta (FP32
// with margin; a superset is harmless) in list order.  32 / L members per
// warp, L lanes each, 4 entries in flight per lane; the mapping is tuned
// for the workload (with the Brownian integrator this search runs every step).
template <int L>
__device__ __forceinline__ void overlap_detect_rows(const Dev& d, const KParams& p, const int* pre,
                                                    int w, int total, int only_rebuilt) {
  constexpr int U = 4, STEP = L * U;
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, sl = lane % L, sub = lane / L;
  const unsigned smask = (L == 32 ? FULL : ((1u << L) - 1u)) << (sub * L);
  const int i = (32 / L) * w + sub;
  const int r = i < total ? row_rank_in(d, pre, i) : 0;
  const int rep = d.rep_of[r];
  const RepConst& R = d.rc[rep];
  const Scalars* sc = d.sc + rep;
  int h = -1, n = 0;
  float4 Pf = make_float4(0.f, 0.f, 0.f, 0.f);
  // rows of replicas whose near entries are current stay as they are
  if (i < total && r - R.base < sc->n_rank && !(only_rebuilt && !sc->rebuild)) h = d.ref[r];
  if (h >= 0) {
    Pf = d.posf[h];
    n = d.nn[h];
  }
  int nmax = n;
#pragma unroll
  for (int o = L; o < 32; o <<= 1) nmax = max(nmax, __shfl_xor_sync(FULL, nmax, o));
  // rc + 2 delta in FP32 (sqrtf is exact to an ulp; the margin covers it)
  const float rn2 = near_radius2(d, p, R);
  const int* row = d.list + (size_t)(h >= 0 ? h : 0) * p.mnb;
  int* near = d.near + (size_t)(h >= 0 ? h : 0) * kNearCap;
  const unsigned lt = (1u << lane) - 1u;
  int cnt = 0;
  bool any = false;
  for (int base = 0; base < nmax; base += STEP) {
    int j[U];
    float4 Q[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int jj = base + L * u + sl;
      j[u] = jj < n ? __ldg(row + jj) : -1;
    }
#pragma unroll
    for (int u = 0; u < U; ++u) Q[u] = j[u] >= 0 ? d.posf[j[u]] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int u = 0; u < U; ++u) {
      bool inc = false;
      if (j[u] >= 0 && elem_of(Q[u]) != 0) {
        float fx, fy, fz;
        vdist_nint_f(R, Pf, Q[u], fx, fy, fz);
        inc = fx * fx + fy * fy + fz * fz <= rn2;
      }
      const unsigned bal = __ballot_sync(FULL, inc) & smask;
      if (inc) {
        const int pos = cnt + __popc(bal & lt);
        if (pos < kNearCap) near[pos] = j[u];
        if (elem_of(Q[u]) != DML_Z_CG) {
          uf_union(d.g, (volatile int*)d.uf, h, j[u]);
          d.active[j[u]] = 1;
        }
      }
      cnt += __popc(bal);
      any = any || bal != 0;
    }
  }
  if (sl == 0 && h >= 0) {
    d.near_count[h] = cnt > kNearCap ? -1 : cnt;
    if (any) d.active[h] = 1;
  }
}

// mode 0: every replica; 1: only if some list was rebuilt since the force
// scan, for the replicas that rebuilt; 2: the replicas that rebuilt.
template <int L>
__global__ void __launch_bounds__(256, 8) overlap_detect_kernel(Dev d, KParams p, int mode) {
  DML_GRID_WAIT();
  if (mode == 1 && !d.g->near_stale) return;  // the force scan found them
  const int nw = gridDim.x * (blockDim.x >> 5);
  // modes 1 and 2 walk only the rows of the replicas that rebuilt
  const int* pre = mode != 0 ? d.reb_pre : d.rank_pre;
  const int total = pre[d.nrep];
  for (int w = warp_id_global(); (32 / L) * w < total; w += nw)
    overlap_detect_rows<L>(d, p, pre, w, total, mode != 0);
}

// Atoms with no near entry are examined trivially in pass 1 (skip = true)
// and can never be moved; the others are counted per component root and
// listed (act_list) for the component passes.  Every lane calls it.
__device__ __forceinline__ void overlap_count_at(Dev d, int n_rank, int rep, int pos) {
  const int lane = threadIdx.x & 31;
  const int h = ref_slot(d, pos, d.rc[rep].base + d.sc[rep].n_slots);
  bool act = false;
  int r = -1;
  if (h >= 0) {
    if (d.active[h]) {
      act = true;
      r = d.rank[h];
    } else {
      d.skip[h] = 1;
    }
  }
  const unsigned m = __ballot_sync(0xffffffffu, act);
  if (!m) return;
  const int leader = __ffs(m) - 1;
  int b = 0;
  if (lane == leader) b = atomicAdd(d.pr_cnt + rep * kCntStride + kCntAct, __popc(m));
  b = __shfl_sync(0xffffffffu, b, leader);
  if (!act) return;
  d.act_list[d.rc[rep].base + b + __popc(m & ((1u << lane) - 1u))] = r;
  int root = uf_find((volatile int*)d.uf, h);
  d.uf[h] = root;
  atomicAdd(&d.comp_size[root], 1);
}

__global__ void overlap_count_kernel(Dev d, int n_rank) {
  DML_GRID_WAIT();
  const int rep = block_rep(d);
  if ((int)blockIdx.x * kSpan >= d.rc[rep].base + d.sc[rep].n_slots) return;
#pragma unroll
  for (int u = 0; u < kSlotU; ++u) overlap_count_at(d, n_rank, rep, span_pos(u));
}

// The prefix of the listed members of the replicas with more than
// kCompBlockMax of them (act_big_pre), one block.
__global__ void overlap_big_prefix_kernel(Dev d) {
  DML_GRID_WAIT();
  __shared__ int s_carry;
  if (threadIdx.x == 0) s_carry = 0;
  __syncthreads();
  for (int r0 = 0; r0 < d.nrep; r0 += blockDim.x) {
    const int r = r0 + threadIdx.x;
    int v = 0;
    if (r < d.nrep) {
      v = d.pr_cnt[r * kCntStride + kCntAct];
      if (v <= kCompBlockMax) v = 0;
    }
    int tot;
    const int e = blk_scan_excl(v, &tot);
    if (r < d.nrep) d.act_big_pre[r] = s_carry + e;
    __syncthreads();
    if (threadIdx.x == 0) s_carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) d.act_big_pre[d.nrep] = s_carry;
}

// The replica of position g of the big replicas' listed members: the last
// replica r with act_big_pre[r] <= g (then act_big_pre[r + 1] > g, so r has
// listed members).
__device__ __forceinline__ int big_rep_of(const Dev& d, int g) {
  int lo = 0, hi = d.nrep - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (d.act_big_pre[mid] <= g) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Component numbers and member ranges for the roots among the listed
// members, one atomic per warp on each counter (the components are
// independent, so their numbering is free).  Per position of each replica's
// list segment; every lane calls it.
__device__ __forceinline__ void overlap_assign_at(const Dev& d, int end, int i,
                                                  int* n_rep_comp = nullptr) {
  const int lane = threadIdx.x & 31;
  int h = -1, sz = 0;
  if (i < end) {
    h = d.ref[d.act_list[i]];
    if (d.uf[h] == h) sz = d.comp_size[h];
  }
  const bool has = sz > 0;
  const unsigned m = __ballot_sync(0xffffffffu, has);
  if (!m) return;
  int x = has ? sz : 0;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  const int total = __shfl_sync(0xffffffffu, x, 31);
  const int leader = __ffs(m) - 1;
  int bc = 0, bt = 0;
  if (lane == leader) {
    bc = atomicAdd(&d.g->n_comp, __popc(m));
    bt = atomicAdd(&d.g->comp_total, total);
    if (n_rep_comp) atomicAdd(n_rep_comp, __popc(m));
  }
  bc = __shfl_sync(0xffffffffu, bc, leader);
  bt = __shfl_sync(0xffffffffu, bt, leader);
  if (has) {
    const int cid = bc + __popc(m & ((1u << lane) - 1u));
    d.comp_id[h] = cid;
    d.comp_list[2 * cid] = bt + x - sz;
    d.comp_list[2 * cid + 1] = sz;
  }
}

// The same bookkeeping for the replicas with more than kCompBlockMax listed
// members, three grid kernels over all of their listed members (the stages
// need every block's results): component numbers and ranges, the members
// scattered, the members in rank order (each member's place is the number
// of smaller ranks in its component).
__global__ void overlap_assign_big_kernel(Dev d) {
  DML_GRID_WAIT();
  const int total = d.act_big_pre[d.nrep];
  const int nw = gridDim.x * (blockDim.x >> 5);
  for (int w = warp_id_global(); 32 * w < total; w += nw) {
    const int g = 32 * w + (threadIdx.x & 31);
    int end = 0, i = 1;  // past the total: no entry
    if (g < total) {
      const int rep = big_rep_of(d, g);
      const int base = d.rc[rep].base;
      end = base + d.pr_cnt[rep * kCntStride + kCntAct];
      i = base + g - d.act_big_pre[rep];
    }
    overlap_assign_at(d, end, i);
  }
}

__device__ __forceinline__ int big_act_entry(const Dev& d, int g) {
  const int rep = big_rep_of(d, g);
  return d.act_list[d.rc[rep].base + g - d.act_big_pre[rep]];
}

__global__ void overlap_scatter_big_kernel(Dev d) {
  DML_GRID_WAIT();
  const int total = d.act_big_pre[d.nrep];
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
    const int r = big_act_entry(d, g);
    const int root = d.uf[d.ref[r]];
    d.comp_rank[d.comp_list[2 * d.comp_id[root]] + atomicAdd(&d.comp_fill[root], 1)] = r;
  }
}

__global__ void overlap_order_big_kernel(Dev d) {
  DML_GRID_WAIT();
  const int total = d.act_big_pre[d.nrep];
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
    const int r = big_act_entry(d, g);
    const int h = d.ref[r];
    const int cid = d.comp_id[d.uf[h]];
    const int off = d.comp_list[2 * cid], sz = d.comp_list[2 * cid + 1];
    const int* rk = d.comp_rank + off;
    int before = 0;
    for (int q = 0; q < sz; ++q) before += rk[q] < r;
    d.comp_members[off + before] = h;
  }
}

// Examination of o1 = x in pass `pass` (dana.F90:871-935).
__device__ void overlap_exam(const Dev& d, const KParams& p, int x, int pass, int* again) {
  const int rep = d.rep_of[x];
  const RepConst& R = d.rc[rep];
  Scalars* sc = d.sc + rep;
  int nc = d.near_count[x];
  int n = nc >= 0 ? nc : d.nn[x];
  const int* src = nc >= 0 ? d.near + (size_t)x * kNearCap : d.list + (size_t)x * p.mnb;
  // x's own position changes only where the walk ends (its near entries
  // never hold x), so it is read once
  const double4 P = d.pos[x];
  const float4 Pf = d.posf[x];
  for (int q = 0; q < n; ++q) {
    int j = src[q];
    if (d.state[j] != ST_LIVE) continue;
    // |P - Q|^2 > rc^2 decided from the FP32 copies outside the margins
    // (a NaN distance takes the FP64 test, as in the reference it passes)
    const float4 Qf = d.posf[j];
    float fx, fy, fz;
    vdist_nint_f(R, Pf, Qf, fx, fy, fz);
    const float df = fx * fx + fy * fy + fz * fz;
    if (df > R.rc_hi2) continue;
    double4 Q = d.pos[j];
    if (!(df < R.rc_lo2)) {
      double vx, vy, vz;
      vdist_nint(R, P, Q, vx, vy, vz);
      double dr = dot3(vx, vy, vz);
      if (dr > p.rc2) continue;
    }
    if (d.typ[j] == DML_Z_CG) {
      count_add(&sc->try_, 1ull);
      double ne = dml_uniform(dml_draw(R.seed, d.g->step, (uint64_t)d.id[x], DML_RNG_OVERLAP,
                                       (uint32_t)pass));
      if (ne < p.prob) {
        count_add(&sc->depo, 1ull);
        d.typ[x] = DML_Z_F;
        note_f(d, x);
        float4 f = d.posf[x];
        f.w = __int_as_float(DML_Z_F);
        d.posf[x] = f;
        if (P.z > sc->z0) raise_error(d.g, DML_E_DENDRITE, x);
      } else {
        double4 O = d.old_cg[x];
        d.pos[x] = O;
        d.posf[x] = to_f4(O, d.typ[x]);
        d.skip[x] = 0;
        d.dirty[x / kSpan] = 1;
      }
      break;
    }
    double4 Oj = d.old_cg[j];
    if (p.reservoir == DML_RESERVOIR_PISTON) {
      double4 Ox = d.old_cg[x];
      bool j_old = Q.x == Oj.x && Q.y == Oj.y && Q.z == Oj.z;
      bool x_old = P.x == Ox.x && P.y == Ox.y && P.z == Ox.z;
      if (j_old && x_old) {
        count_add(&sc->choques3, 1ull);
        continue;
      }
    }
    d.pos[j] = Oj;
    d.posf[j] = to_f4(Oj, d.typ[j]);
    d.dirty[j / kSpan] = 1;
    d.acel[j] = make_double4(0.0, 0.0, 0.0, 0.0);
    d.vel[j] = make_double4(0.0, 0.0, 0.0, 0.0);
    d.skip[j] = 0;
    count_add(&sc->choques, 1ull);
    *again = 1;
  }
}

// One thread per component, members in rank order.  With
// `all_passes` (prob >= 1: a contact capture never fails, so no atom is left
// with skip = false unless an ion was moved back in its own component) the
// component runs every pass itself: pass p of the reference examines exactly
// the members with skip = false, in rank order, whatever the other
// components do.  Otherwise only pass 1 runs here and the later passes run
// in overlap_passn_kernel with a barrier per pass.
__device__ void overlap_pass1_comp(const Dev& d, const KParams& p, int all_passes, int cid) {
  int off = d.comp_list[2 * cid], sz = d.comp_list[2 * cid + 1];
  const int* mem = d.comp_members + off;
  int pass = 1;
  for (;;) {
    int again = 0;
    for (int i = 0; i < sz; ++i) {
      int x = mem[i];
      if (d.skip[x]) continue;
      d.skip[x] = 1;
      overlap_exam(d, p, x, pass, &again);
    }
    if (!all_passes) {
      if (again) {
        d.sc[d.rep_of[mem[0]]].again2 = 1;
        d.g->again = 1;
      }
      return;
    }
    if (!again) break;
    if (pass >= p.max_passes) {
      raise_error(d.g, DML_E_OVERLAP_PASSES, pass + 1);
      break;
    }
    pass += 1;
  }
  if (sz > 0) atomicMax(&d.sc[d.rep_of[mem[0]]].passes, pass);
  atomicMax(&d.g->passes, pass);
}

// The bookkeeping of one replica's listed members (component numbers and
// ranges, members scattered, members in rank order), then, when every pass
// can run inside a component (prob >= 1) and the replica has at most one
// component per thread, the component passes: one block per replica, the
// stages separated by block barriers (a component lies inside one replica).
// A replica with more components leaves its passes to overlap_pass1_kernel,
// whose grid spreads them over every SM (comp_defer); one with more than
// kCompBlockMax listed members was handled by the _big kernels.
__global__ void overlap_comp_kernel(Dev d, KParams p, int passes) {
  DML_GRID_WAIT();
  const int rep = blockIdx.x;
  const int base = d.rc[rep].base;
  const int end = base + d.pr_cnt[rep * kCntStride + kCntAct];
  if (end == base) return;  // no member with a near contact
  if (end - base > kCompBlockMax) {
    if (threadIdx.x == 0) d.sc[rep].comp_defer = passes;
    return;
  }
  __shared__ int s_ncomp;
  if (threadIdx.x == 0) s_ncomp = 0;
  __syncthreads();
  for (int i0 = base; i0 < end; i0 += blockDim.x)
    overlap_assign_at(d, end, i0 + threadIdx.x, &s_ncomp);
  __syncthreads();
  const bool here = passes && s_ncomp <= (int)blockDim.x;
  if (threadIdx.x == 0) d.sc[rep].comp_defer = passes && !here;
  for (int i = base + threadIdx.x; i < end; i += blockDim.x) {
    const int h = d.ref[d.act_list[i]];
    const int root = d.uf[h];
    const int cid = d.comp_id[root];
    d.comp_rank[d.comp_list[2 * cid] + atomicAdd(&d.comp_fill[root], 1)] = d.act_list[i];
  }
  __syncthreads();
  for (int i = base + threadIdx.x; i < end; i += blockDim.x) {
    const int r = d.act_list[i];
    const int h = d.ref[r];
    const int cid = d.comp_id[d.uf[h]];
    const int off = d.comp_list[2 * cid], sz = d.comp_list[2 * cid + 1];
    const int* rk = d.comp_rank + off;
    int before = 0;
    for (int q = 0; q < sz; ++q) before += rk[q] < r;
    d.comp_members[off + before] = h;
  }
  if (!here) return;
  __syncthreads();
  // every component of the replica once: through its root's listed member
  for (int i = base + threadIdx.x; i < end; i += blockDim.x) {
    const int h = d.ref[d.act_list[i]];
    if (d.uf[h] == h) overlap_pass1_comp(d, p, 1, d.comp_id[h]);
  }
}

// Pass 1 of every component on a fixed grid; with all_passes (prob >= 1)
// every pass, and only the components of replicas that overlap_comp_kernel
// left to this kernel.
__global__ void overlap_pass1_kernel(Dev d, KParams p, int all_passes) {
  DML_GRID_WAIT();
  const int ncomp = d.g->n_comp;
  for (int cid = blockIdx.x * blockDim.x + threadIdx.x; cid < ncomp;
       cid += gridDim.x * blockDim.x) {
    if (all_passes) {
      const int sz = d.comp_list[2 * cid + 1];
      if (sz == 0 || !d.sc[d.rep_of[d.comp_members[d.comp_list[2 * cid]]]].comp_defer) continue;
    }
    overlap_pass1_comp(d, p, all_passes, cid);
  }
}

// Passes 2.. (the recursion, needed when a capture can fail): one block, a
// barrier between passes.  Each replica recurses on its own flag, as it would
// alone: a component is examined in pass p only if its replica's pass p-1
// moved an atom.
__global__ void overlap_passn_kernel(Dev d, KParams p) {
  DML_GRID_WAIT();
  __shared__ int again_s;
  __shared__ int go;
  int ncomp = d.g->n_comp;
  int pass = 1;
  if (threadIdx.x == 0) go = d.g->again;
  __syncthreads();
  while (go) {
    pass += 1;
    for (int r = threadIdx.x; r < d.nrep; r += blockDim.x) {
      d.sc[r].again = d.sc[r].again2;
      d.sc[r].again2 = 0;
      if (d.sc[r].again) d.sc[r].passes = pass;
    }
    if (pass > p.max_passes) {
      if (threadIdx.x == 0) raise_error(d.g, DML_E_OVERLAP_PASSES, pass);
      break;
    }
    if (threadIdx.x == 0) again_s = 0;
    __syncthreads();
    int again_any = 0;
    for (int cid = threadIdx.x; cid < ncomp; cid += blockDim.x) {
      int off = d.comp_list[2 * cid], sz = d.comp_list[2 * cid + 1];
      const int* mem = d.comp_members + off;
      if (sz == 0) continue;
      Scalars* sc = d.sc + d.rep_of[mem[0]];
      if (!sc->again) continue;
      int again = 0;
      for (int i = 0; i < sz; ++i) {
        int x = mem[i];
        if (d.skip[x]) continue;
        d.skip[x] = 1;
        overlap_exam(d, p, x, pass, &again);
      }
      if (again) {
        sc->again2 = 1;
        again_any = 1;
      }
    }
    if (again_any) atomicOr(&again_s, 1);
    __syncthreads();
    if (threadIdx.x == 0) go = again_s;
    __syncthreads();
  }
  if (threadIdx.x == 0) d.g->passes = pass;
}

// ------------------------------------------------- capture commit, rho, piston
// dana.F90:228-236: every F member of hs%ref becomes CG and leaves hs%ref
// (its rank becomes a hole; the order of the remaining members is kept).
__device__ __forceinline__ void commit_at(Dev d, int h) {
  const int rep = d.rep_of[h];
  Scalars* sc = d.sc + rep;
  const int r = d.rank[h];
  if (r < 0 || d.typ[h] != DML_Z_F) return;
  if (atomicCAS(&d.rank[h], r, -1) != r) return;  // listed twice: once only
  d.typ[h] = DML_Z_CG;
  float4 f = d.posf[h];
  f.w = __int_as_float(DML_Z_CG);
  d.posf[h] = f;
  d.ref[r] = -1;
  atomicSub(&sc->n_ref, 1);
  atomicAdd(&sc->n_new_cg, 1);
  if (d.in_gcmc[h]) {  // gcmc%detach (dana.F90:235)
    d.in_gcmc[h] = 0;
    d.gorder[d.gpos[h]] = -1;
    atomicSub(&sc->n_gcmc, 1);
  }
}

// Over the atoms that became F since the last commit (listed where the
// element is set: atom_pbc, overlap_moveback's contact capture, loading and
// chunk attachment), one block: captures are few, and the block empties
// the list when it is done.
__global__ void commit_kernel(Dev d) {
  DML_GRID_WAIT();
  const int n = min(d.g->n_f, d.cap);
  for (int q = threadIdx.x; q < n; q += blockDim.x) commit_at(d, d.flist[q]);
  __syncthreads();
  if (threadIdx.x == 0) d.g->n_f = 0;
}

// calc_rho (dana.F90:521-549): integer count, so any reduction order is exact.
__global__ void calc_rho_kernel(Dev d, KParams p, int n_slots) {
  DML_GRID_WAIT();
  // grids are sized by capacity; the block's replica gives the live count
  const int rep = block_rep(d);
  const RepConst& R = d.rc[rep];
  Scalars* sc = d.sc + rep;
  n_slots = R.base + sc->n_slots;  // positions in use end here
  // the spans in use take part (the first one always); a block past them
  // leaves at once
  const int nu = max(1, (n_slots - R.base + kSpan - 1) / kSpan);
  if ((int)blockIdx.x - R.base / kSpan >= nu) return;
  double z0 = sc->z0;
  double zt = p.ztop_is_z1 != 0.0 ? sc->z1 : sc->zmax;
  // z > z0 && z < zt from the FP32 copy zf = RN32(z) (monotone rounding:
  // zf beyond RN32 of a bound decides), FP64 when zf equals one (or NaN);
  // a slot is live exactly when its FP32 copy carries an element.  The
  // bounds' FP32 copies are formed once per block (conversions issue on the
  // narrow FP64 pipe).
  __shared__ float s_z0f, s_ztf;
  if (threadIdx.x == 0) {
    s_z0f = (float)z0;
    s_ztf = (float)zt;
  }
  __syncthreads();
  const float z0f = s_z0f, ztf = s_ztf;
  const bool used = (int)blockIdx.x * kSpan < n_slots;
  float4 Pf[kSlotU];
#pragma unroll
  for (int u = 0; u < kSlotU; ++u) {
    const int s = span_pos(u);
    Pf[u] = used && s < n_slots ? d.posf[s] : make_float4(0.f, 0.f, 0.f, 0.f);
  }
  int c = 0;
#pragma unroll
  for (int u = 0; u < kSlotU; ++u) {
    if (elem_of(Pf[u]) == 0) continue;
    const float zf = Pf[u].z;
    if (zf > z0f && zf < ztf) {
      c += 1;
    } else if (!(zf < z0f || zf > ztf)) {
      const double z = d.pos[span_pos(u)].z;
      c += (z > z0 && z < zt) ? 1 : 0;
    }
  }
  for (int off = 16; off > 0; off >>= 1) c += __shfl_down_sync(0xffffffffu, c, off);
  __shared__ int s_c;
  if (threadIdx.x == 0) s_c = 0;
  __syncthreads();
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(&s_c, c);
  __syncthreads();
  c = s_c;
  __shared__ bool last;
  if (threadIdx.x == 0) {
    if (c) atomicAdd(&sc->rho_count, c);
    __threadfence();
    unsigned t = atomicAdd(&sc->ticket2, 1u);
    last = (t == (unsigned)nu - 1u);  // the replica's last block
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    __threadfence();
    int g = atomicAdd(&sc->rho_count, 0);
    double vol = R.box[0] * R.box[1] * (zt - z0);
    sc->rho = (double)g / vol;
    sc->rho_count = 0;
    sc->ticket2 = 0;
  }
}

// maxz (dana.F90:776-794).  lohi is formed once per block (an FP64 divide
// issues on the narrow FP64 pipe; every thread forming it cost more than
// the compression itself).
__device__ __forceinline__ void piston_at(Dev d, KParams p, int n_slots, int rep, int pos,
                                          double lohi) {
  const RepConst& R = d.rc[rep];
  Scalars* sc = d.sc + rep;
  n_slots = R.base + sc->n_slots;  // positions in use end here
  const int s = pos;
  const double z0 = sc->z0;
  // A slot is live exactly when its FP32 copy carries an element, and
  // RN32(z) < RN32(z0) implies z < z0 (monotone rounding): only atoms at or
  // above RN32(z0) read their FP64 z.  Only z changes, so the copy keeps its
  // x, y and element.
  if (s < n_slots) {
    float4 f = d.posf[s];
    if (elem_of(f) != 0 && !(f.z < (float)z0)) {
      double* const pz = reinterpret_cast<double*>(d.pos + s) + 2;
      const double z = *pz;
      if (z > z0) {
        const double zn = z - lohi * (z - z0);
        *pz = zn;
        f.z = f64_to_f32_rn(zn);
        d.posf[s] = f;
      }
    }
  }
  if (s == R.base) {
    double zm = sc->zmax;
    sc->zmax_frame = zm;
    sc->lohi = lohi;
    sc->zmax = zm - lohi * (zm - z0);
  }
}

__global__ void piston_kernel(Dev d, KParams p, int n_slots) {
  DML_GRID_WAIT();
  const int rep = block_rep(d);
  __shared__ double s_lohi;
  if (threadIdx.x == 0) {
    const Scalars* sc = d.sc + rep;
    s_lohi = (p.h_over_tau * ((sc->rho0 - sc->rho) / sc->rho));
  }
  __syncthreads();
  const double lohi = s_lohi;
#pragma unroll
  for (int u = 0; u < kSlotU; ++u) piston_at(d, p, n_slots, rep, span_pos(u), lohi);
}


// ------------------------------------------------------------- bloques
// cgroup_tessellate (Cells.F90:180-265) after the box height changed to bz:
// a tessellated replica keeps its cell counts while every cell edge stays
// in (rc + skin, (n + 1)/n (rc + skin)], else the counts are taken again
// from int(box / (rc + skin)); cells are off while all three counts are
// below 4.  Only z changes (the chunk reservoir raises the box), so the x
// and y values are those of the replica's creation.
__device__ void tessellate_height(RepConst& R, const KParams& p, double bz) {
  R.box[2] = bz;
  R.one_box[2] = 1.0 / bz;
  R.halfbox[2] = bz * .5;
  R.boxf[2] = __double2float_rn(bz);
  R.halfboxf[2] = __double2float_rn(bz * .5);
  bool keep = false;
  if (R.use_cells) {
    keep = true;
    for (int k = 0; k < 3; ++k) {
      if (!((double)(R.ncells[k] + 1) >= R.box[k] / p.rcut_b)) keep = false;
      if (!(p.rcut_b < R.box[k] / (double)R.ncells[k])) keep = false;
    }
  }
  if (!keep) {
    int n[3];
    for (int k = 0; k < 3; ++k) n[k] = (int)(R.box[k] / p.rcut_b);
    if (n[0] < 4 && n[1] < 4 && n[2] < 4) return;  // still no cells
    R.use_cells = 1;
    for (int k = 0; k < 3; ++k) R.ncells[k] = n[k] < 1 ? 1 : n[k];
  }
  for (int k = 0; k < 3; ++k) {
    R.cell[k] = R.box[k] / (double)R.ncells[k];
    R.inv_cellf[k] = __double2float_rn(1.0 / R.cell[k]);
    R.cellf[k] = __double2float_rn(R.cell[k]);
    R.head_dim[k] = R.ncells[k] + 2;
  }
  R.ncell = R.head_dim[0] * R.head_dim[1] * R.head_dim[2];
  R.tess_hif = __double2float_rn((double)(R.ncells[2] + 1) * R.cell[2]);
}

// bloques (dana.F90:716-773), one block per replica, one thread: when the
// sensor density strays from rhomedia by 0.186 rhomedia or more (the
// literal is single precision), the planes rise by the chunk height, the
// template atoms are attached in template order (sys%alist appended, first
// free hs and hs%b slots, hs%ref appended, a new id; atom_asign copies the
// template's position, old position, velocity, acceleration, force, energy
// and element), the template rises, the box height becomes zmax and the
// list is marked stale, so that the test_update after it rebuilds.
__global__ void bloques_kernel(Dev d, KParams p) {
  DML_GRID_WAIT();
  const int rep = blockIdx.x;
  if (threadIdx.x != 0) return;
  Scalars* sc = d.sc + rep;
  RepConst& R = d.rc[rep];
  const double drho = sc->rho - p.rhomedia;
  if (fabs(drho) < (p.rhomedia * (double)0.186f)) return;
  sc->z0 = sc->z0 + p.chunk_dist;
  sc->z1 = sc->z1 + p.chunk_dist;
  sc->zmax = sc->zmax + p.chunk_dist;
  sc->zmax_frame = sc->zmax;
  sc->listed = 0;
  const int B = R.base;
  double4* tp = d.chk_pos + (size_t)rep * p.n_chunk;
  double4* to = d.chk_pold + (size_t)rep * p.n_chunk;
  for (int j = 0; j < p.n_chunk; ++j) {
    // first free hs slot (limbo slots are not free) and hs%b slot
    const int nat = sc->n_atoms + 1, bnat = sc->b_nat + 1;
    const int ns = sc->n_slots, nb = sc->n_b;
    int ls = ns, lb = nb;
    if (ns >= nat + sc->nlimbo) {
      ls = INT_MAX;
      for (int q = sc->free_lo; q < ns; ++q)
        if (d.state[B + q] == ST_NULL) {
          ls = q;
          break;
        }
    }
    if (nb >= bnat) {
      lb = INT_MAX;
      for (int q = sc->bfree_lo; q < nb; ++q)
        if (d.b2hs[B + q] < 0) {
          lb = q;
          break;
        }
    }
    if (ls == INT_MAX || lb == INT_MAX) {
      raise_error(d.g, DML_E_INDEX, j);
      return;
    }
    if (ls >= R.cap || lb >= R.cap || sc->n_rank >= R.cap || sc->n_alist >= R.cap) {
      raise_error(d.g, DML_E_CAPACITY, j);
      return;
    }
    const int slot = B + ls, bs = B + lb;
    const int typ = d.chk_typ[j];
    const double4 P = tp[j], O = to[j];
    d.pos[slot] = P;
    d.pos_old[slot] = O;
    d.posf[slot] = to_f4(P, typ);
    d.posf_old[slot] = to_f4(O, 0);
    d.vel[slot] = make_double4(0.0, 0.0, 0.0, 0.0);
    d.acel[slot] = make_double4(0.0, 0.0, 0.0, 0.0);
    d.force[slot] = make_double4(0.0, 0.0, 0.0, 0.0);
    d.epot[slot] = 0.0;
    d.old_cg[slot] = make_double4(1e8, 1e8, 1e8, 0.0);
    d.typ[slot] = (int8_t)typ;
    d.skip[slot] = 0;
    d.id[slot] = sc->next_id;
    sc->next_id += 1;
    d.ev_count[slot] = 0;
    d.nn[slot] = 0;
    if (typ == DML_Z_F) note_f(d, slot);
    // sys
    const int ap = sc->n_alist;
    d.alist[B + ap] = slot;
    d.apos[slot] = B + ap;
    sc->n_alist = ap + 1;
    // hs%ref
    const int rk = sc->n_rank;
    d.ref[B + rk] = slot;
    d.rank[slot] = B + rk;
    sc->n_rank = rk + 1;
    sc->n_ref += 1;
    // hs%b (not sorted into cells: the list is stale)
    d.b2hs[bs] = slot;
    d.bslot[slot] = bs;
    if (lb == nb) sc->n_b = nb + 1;
    sc->b_nat = bnat;
    sc->bfree_lo = lb + 1;
    // hs
    d.state[slot] = ST_LIVE;
    if (ls == ns) sc->n_slots = ns + 1;
    sc->free_lo = ls + 1;
    sc->n_atoms = nat;
    // the template rises (dana.F90:762-763)
    tp[j].z = P.z + p.chunk_dist;
    to[j].z = O.z + p.chunk_dist;
  }
  tessellate_height(R, p, sc->zmax);
  atomicOr(&d.g->chunk_event, 1);
}

__global__ void chunk_cond_kernel(Global* g, cudaGraphConditionalHandle h) {
  DML_GRID_WAIT();
  cudaGraphSetConditional(h, g->chunk_event ? 1u : 0u);
}

// ------------------------------------------------------------------ gcmc_run
// gcmc_run (dana.F90:590-713): the trials are sequential (each sees the
// previous one's insertion or deletion), so one block of 1024 threads runs
// them in order and parallelises inside a trial: the hard-core test over the
// gcmc group, the m-th in-slab selection, the first-free slot searches
// (igroup_attach_atom, Groups.F90:1083-1093), the new atom's own list
// (ngroup_cells_atom over chains that hold this run's insertions at their
// heads, Cells.F90:299-300) and its appends to the other lists
// (ngroup_sort_atom, Neighbor.F90:271-318).


// First index in [lo, hi) where pred holds, or INT_MAX; every thread of the
// block calls it (the result lands in *s_res and is returned to all).  Each
// thread tests 8 strided indices per round, so the loads of a round are
// independent and a round covers 8 * blockDim.x indices.
template <class Pred>
__device__ int blk_find_first(int lo, int hi, Pred pred, int* s_res) {
  if (threadIdx.x == 0) *s_res = INT_MAX;
  __syncthreads();
  for (int base = lo; base < hi; base += 8 * (int)blockDim.x) {
    int best = INT_MAX;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      int i = base + k * (int)blockDim.x + (int)threadIdx.x;
      if (i < hi && pred(i)) best = min(best, i);
    }
    if (best != INT_MAX) atomicMin(s_res, best);
    if (__syncthreads_or(best != INT_MAX)) break;
  }
  int r = *s_res;
  __syncthreads();
  return r;
}

// Stable in-place compaction of an order array (holes = -1); pos_of[h]
// receives the new position of every member.
__device__ int blk_compact(int* arr, int off, int n, int* pos_of) {
  int out = 0;
  for (int base = 0; base < n; base += blockDim.x) {
    int i = base + threadIdx.x;
    int h = i < n ? arr[off + i] : -1;
    int tot;
    int pre = blk_scan_excl(h >= 0 ? 1 : 0, &tot);
    __syncthreads();
    if (h >= 0) {
      arr[off + out + pre] = h;
      pos_of[h] = off + out + pre;
    }
    out += tot;
    __syncthreads();
  }
  for (int i = out + threadIdx.x; i < n; i += blockDim.x) arr[off + i] = -1;
  __syncthreads();
  return out;
}

__device__ __forceinline__ bool list_entry_in(const KParams& p, const RepConst& R, double4 a,
                                              double4 b, bool strict) {
  double vx, vy, vz;
  vdist_nint(R, a, b, vx, vy, vz);
  double rd = dot3(vx, vy, vz);
  return strict ? rd < p.rlist2 : !(rd > p.rlist2);
}

// Own list of a newly attached atom i, one warp (ngroup_cells_atom,
// Neighbor.F90:550-603, or ngroup_verlet_atom :426-463).
__device__ void gcmc_own_list(const Dev& d, const KParams& p, const RepConst& R, int i, int nb_loc) {
  int lane = threadIdx.x & 31;
  double4 P = d.pos[i];
  int* row = d.list + (size_t)i * p.mnb;
  int cnt = 0;
  if (R.use_cells) {
    int rc[3] = {cell_index(P.x, R.cell[0]), cell_index(P.y, R.cell[1]), cell_index(P.z, R.cell[2])};
    for (int nabor = 0; nabor < 27; ++nabor) {
      int nc[3];
      for (int k = 0; k < 3; ++k) {
        int t = map_off(nabor, k) + rc[k] - 1;
        t = (t + R.ncells[k]) % R.ncells[k];
        nc[k] = t + 1;
      }
      int c = R.cell_off + (nc[2] * R.head_dim[1] + nc[1]) * R.head_dim[0] + nc[0];
      // atoms inserted during this run, most recent first (chain heads)
      if (lane == 0) {
        for (int j = d.ins_head[c]; j >= 0; j = d.ins_next[j]) {
          if (j == i || d.state[j] != ST_LIVE) continue;
          if (list_entry_in(p, R, d.pos[j], P, true)) {
            if (cnt < p.mnb) row[cnt] = j;
            ++cnt;
          }
        }
      }
      cnt = __shfl_sync(0xffffffffu, cnt, 0);
      int start = d.cell_start[c];
      int num = d.cell_start[c + 1] - start;
      for (int base = 0; base < num; base += 32) {
        int idx = base + lane;
        bool inc = false;
        int j = -1;
        if (idx < num) {
          j = d.cell_atoms[start + idx];
          if (j != i && d.state[j] == ST_LIVE) inc = list_entry_in(p, R, d.pos[j], P, true);
        }
        unsigned bal = __ballot_sync(0xffffffffu, inc);
        int pre = __popc(bal & ((1u << lane) - 1u));
        if (inc && cnt + pre < p.mnb) row[cnt + pre] = j;
        cnt += __popc(bal);
      }
    }
  } else {
    int n_b = R.base + nb_loc;
    for (int base = R.base; base < n_b; base += 32) {
      int b = base + lane;
      bool inc = false;
      int j = -1;
      if (b < n_b) {
        j = d.b2hs[b];
        if (j >= 0 && j != i) inc = list_entry_in(p, R, P, d.pos[j], false);
      }
      unsigned bal = __ballot_sync(0xffffffffu, inc);
      int pre = __popc(bal & ((1u << lane) - 1u));
      if (inc && cnt + pre < p.mnb) row[cnt + pre] = j;
      cnt += __popc(bal);
    }
  }
  if (lane == 0) {
    if (cnt > p.mnb) raise_error(d.g, DML_E_NEIGH_OVERFLOW, i);
    d.nn[i] = cnt > p.mnb ? p.mnb : cnt;
    list_new_row(d, i);  // an inserted atom's row, written between full force scans
  }
}

constexpr int kGcmcThreads = 256;
constexpr int kGcmcTrialBatch = 256;  // trials drawn ahead into shared memory

__device__ __forceinline__ bool in_slab(double z, double z0, double zmax) {
  return !(z < z0) && !(z > zmax);
}

// gcmc_run's preparation, one block per replica: the order arrays grow by
// appends (insertions) and gain holes (deletions, captures); they are
// compacted, order kept, before they could overflow and whenever holes make
// up an eighth of them (every per-rank kernel walks the holes too: without
// this, config 5's hs%ref order doubles in length within a few hundred
// steps, and so does the time of those kernels); the listing of
// gcmc_bin_kernel starts empty, the member bounds at their identities, and
// the bit words past the used gcmc%alist positions (appends set bits there)
// are cleared.
__global__ void gcmc_prep_kernel(Dev d, KParams p, int par) {
  DML_GRID_WAIT();
  const int rep = blockIdx.x;
  const RepConst& R = d.rc[rep];
  Scalars* const sc = d.sc + rep;
  const int B = R.base, tid = threadIdx.x, nt = blockDim.x;
  if (tid == 0) d.pr_cnt[rep * kCntStride + kCntGlist] = 0;
  if (!sc->listed) return;  // gcmc_kernel reports the state error
  if (sc->n_rank + p.nadj >= R.cap || 8 * (sc->n_rank - sc->n_ref) > sc->n_rank) {
    int n = blk_compact(d.ref, B, sc->n_rank, d.rank);
    if (tid == 0) sc->n_rank = n;
    __syncthreads();
  }
  if (sc->n_alist + p.nadj >= R.cap || 8 * (sc->n_alist - sc->n_atoms) > sc->n_alist) {
    int n = blk_compact(d.alist, B, sc->n_alist, d.apos);
    if (tid == 0) sc->n_alist = n;
    __syncthreads();
  }
  if (sc->n_gorder + p.nadj >= R.cap || 8 * (sc->n_gorder - sc->n_gcmc) > sc->n_gorder) {
    int n = blk_compact(d.gorder, B, sc->n_gorder, d.gpos);
    if (tid == 0) sc->n_gorder = n;
    __syncthreads();
  }
  if (!par) return;
  const int ng = sc->n_gorder;
  GcmcRepPre* const gr = d.grp + rep;
  if (tid == 0) {
    gr->first = INT_MAX;
    gr->last = -1;
    gr->n_in = 0;
    gr->ng = ng;
  }
  unsigned* wm = d.gw_mem + B / 32;
  unsigned* wsl = d.gw_slab + B / 32;
  const int w0 = (ng + 31) >> 5, w1 = min((ng + p.nadj + 64) >> 5, R.cap >> 5);
  for (int w = w0 + tid; w < w1; w += nt) {
    wm[w] = 0u;
    wsl[w] = 0u;
  }
}

// in_slab(z) of an atom from z's FP32 copy zf = RN32(z): rounding is
// monotone, so zf beyond RN32 of a bound decides the comparison; zf equal to
// it (or NaN) takes the FP64 coordinate.
__device__ __forceinline__ bool in_slab_at(const Dev& d, int h, float zf, float z0f, float zmaxf,
                                           double z0, double zmax) {
  if (zf > z0f && zf < zmaxf) return true;
  if (zf < z0f || zf > zmaxf) return false;
  return in_slab(d.pos[h].z, z0, zmax);
}

// gcmc_run's cell sort, binning pass: every live atom's cell (coalesced
// over hs slots, so no gather), the range check and the halo flag of
// cgroup_sort_atom (Cells.F90:281-302) for all, and a list entry (hs slot,
// cell; with the parallel trials also the FP32 position) for the atoms of
// the z layers the trials can reach.
__device__ __forceinline__ void gcmc_bin_at(const Dev& d, int rep, int pos, int par) {
  const RepConst& R = d.rc[rep];
  Scalars* sc = d.sc + rep;
  const int s = pos;
  const int lane = threadIdx.x & 31;
  int lin = -1;
  // a slot is live exactly when its FP32 copy carries an element
  const float4 Pf = R.use_cells && s < R.base + sc->n_slots ? d.posf[s]
                                                             : make_float4(0.f, 0.f, 0.f, 0.f);
  if (elem_of(Pf) != 0) {
    int c1, c2, c3;
    cell_index3(R, Pf, d.pos + s, c1, c2, c3);
    if (c1 < 0 || c2 < 0 || c3 < 0 || c1 > R.ncells[0] + 1 || c2 > R.ncells[1] + 1 ||
        c3 > R.ncells[2] + 1) {
      raise_error(d.g, DML_E_OUT_OF_TESSELLATION, s);
    } else {
      // the 27-cell stencil never visits the halo: trials fall back to full scans
      if (c1 == 0 || c2 == 0 || c3 == 0 || c1 > R.ncells[0] || c2 > R.ncells[1] ||
          c3 > R.ncells[2])
        sc->halo = 1;
      if (R.gl_all || ((R.gl_cmask >> c3) & 1ull))
        lin = R.cell_off + (c3 * R.head_dim[1] + c2) * R.head_dim[0] + c1;
    }
  }
  const bool in = lin >= 0;
  const unsigned m = __ballot_sync(0xffffffffu, in);
  if (!m) return;
  const int leader = __ffs(m) - 1;
  int b = 0;
  if (lane == leader) b = atomicAdd(d.pr_cnt + rep * kCntStride + kCntGlist, __popc(m));
  b = __shfl_sync(0xffffffffu, b, leader);
  if (!in) return;
  const int at = R.base + b + __popc(m & ((1u << lane) - 1u));
  d.glist[at] = make_int2(s, lin);
  if (par) d.glp[at] = make_float4(Pf.x, Pf.y, Pf.z, __int_as_float(s));
}

// The membership and in-slab bits of the gcmc%alist positions [0, ng) for
// the parallel trials (one word per warp: positions of a warp are 32
// aligned consecutive ones), the first and last member and the
// control-volume count (dana.F90:601-606), reduced over the block.
__device__ __forceinline__ void gcmc_member_words(const Dev& d, int rep) {
  const RepConst& R = d.rc[rep];
  const Scalars* sc = d.sc + rep;
  GcmcRepPre* const gr = d.grp + rep;
  const int B = R.base, lane = threadIdx.x & 31;
  const int ng = gr->ng;
  __shared__ int s_lo, s_hi, s_cnt;
  if (threadIdx.x == 0) {
    s_lo = INT_MAX;
    s_hi = -1;
    s_cnt = 0;
  }
  __syncthreads();
  if ((int)blockIdx.x * kSpan - B < ng) {
    const double z0 = sc->z0, zmax = sc->zmax;
    const float z0f = (float)z0, zmaxf = (float)zmax;
    int h[kSlotU];
#pragma unroll
    for (int u = 0; u < kSlotU; ++u) {
      const int i = span_pos(u) - B;
      h[u] = i < ng ? d.gorder[B + i] : -1;
    }
    float zf[kSlotU];
#pragma unroll
    for (int u = 0; u < kSlotU; ++u) zf[u] = h[u] >= 0 ? d.posf[h[u]].z : 0.0f;
    int lo = INT_MAX, hi = -1, cnt = 0;
#pragma unroll
    for (int u = 0; u < kSlotU; ++u) {
      const int i = span_pos(u) - B;
      const bool mem = h[u] >= 0;
      const bool in = mem && in_slab_at(d, h[u], zf[u], z0f, zmaxf, z0, zmax);
      const unsigned bm = __ballot_sync(0xffffffffu, mem);
      const unsigned bs = __ballot_sync(0xffffffffu, in);
      if (lane == 0 && i < ng) {
        d.gw_mem[(B + i) >> 5] = bm;
        d.gw_slab[(B + i) >> 5] = bs;
      }
      if (bm) {
        lo = min(lo, i - lane + __ffs(bm) - 1);
        hi = max(hi, i - lane + 31 - __clz(bm));
      }
      cnt += __popc(bs);
    }
    if (lane == 0 && hi >= 0) {
      atomicMin(&s_lo, lo);
      atomicMax(&s_hi, hi);
      atomicAdd(&s_cnt, cnt);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && s_hi >= 0) {
    atomicMin(&gr->first, s_lo);
    atomicMax(&gr->last, s_hi);
    atomicAdd(&gr->n_in, s_cnt);
  }
}

__global__ void __launch_bounds__(kBlock, 6) gcmc_bin_kernel(Dev d, int par) {
  DML_GRID_WAIT();
  const int rep = block_rep(d);
  if (blockIdx.x == 0 && threadIdx.x == 0) d.g->n_big = 0;  // cell_order's list
  // a block past the slots in use (and, with the parallel trials, past the
  // gcmc%alist positions in use) has nothing to bin or to mark
  const int lim = max(d.sc[rep].n_slots, par ? d.grp[rep].ng : 0);
  if ((int)blockIdx.x * kSpan - d.rc[rep].base >= lim) return;
#pragma unroll
  for (int u = 0; u < kSlotU; ++u) gcmc_bin_at(d, rep, span_pos(u), par);
  if (par) gcmc_member_words(d, rep);
}

// The same two passes, one block per replica (the parallel trials: most
// replicas leave at once).
__global__ void gcmc_count_rep_kernel(Dev d) {
  DML_GRID_WAIT();
  const int rep = blockIdx.x;
  if (!gcmc_sorts(d, rep, 1)) return;
  const int B = d.rc[rep].base, end = B + d.pr_cnt[rep * kCntStride + kCntGlist];
  for (int i = B + threadIdx.x; i < end; i += blockDim.x) atomicAdd(&d.cell_count[d.glist[i].y], 1);
}

__global__ void gcmc_scatter_rep_kernel(Dev d) {
  DML_GRID_WAIT();
  const int rep = blockIdx.x;
  if (!gcmc_sorts(d, rep, 1)) return;
  const int B = d.rc[rep].base, end = B + d.pr_cnt[rep * kCntStride + kCntGlist];
  for (int i = B + threadIdx.x; i < end; i += blockDim.x) {
    const int2 e = d.glist[i];
    d.cell_atoms[d.cell_start[e.y] + atomicAdd(&d.cell_fill[e.y], 1)] = d.bslot[e.x];
  }
}

// The cell counts of the sequentially run replicas' listed atoms.
__global__ void gcmc_count_kernel(Dev d, int par) {
  DML_GRID_WAIT();
  const int rep = block_rep(d);
  if (!gcmc_sorts(d, rep, par)) return;
  const int end = d.rc[rep].base + d.pr_cnt[rep * kCntStride + kCntGlist];
#pragma unroll
  for (int u = 0; u < kSlotU; ++u) {
    const int i = span_pos(u);
    if (i < end) atomicAdd(&d.cell_count[d.glist[i].y], 1);
  }
}

// Scatter pass over each sorting replica's listed atoms (cell_atoms holds
// hs%b slots until cell_order turns them into hs slots).
__global__ void gcmc_scatter_kernel(Dev d, int par) {
  DML_GRID_WAIT();
  const int rep = block_rep(d);
  if (!gcmc_sorts(d, rep, par)) return;
  const int end = d.rc[rep].base + d.pr_cnt[rep * kCntStride + kCntGlist];
#pragma unroll
  for (int u = 0; u < kSlotU; ++u) {
    const int i = span_pos(u);
    if (i < end) {
      const int2 e = d.glist[i];
      d.cell_atoms[d.cell_start[e.y] + atomicAdd(&d.cell_fill[e.y], 1)] = d.bslot[e.x];
    }
  }
}


// One trial of gcmc_run: its uniforms (coin, acceptance, the three
// coordinates, the pick) and trial point, drawn before the trials run.
struct GcmcTrial {
  double coin, uacc, upick;
  double4 r;   // trial point (x, y, z)
  float4 rf;   // its FP32 copy
};

// Linear index of stencil cell `nabor` (map order) around the point's cell.
// Stencil cell `nabor` (map order) of the interior cell (t1, t2, t3), with
// the periodic wrap of cell_pbc.
__device__ __forceinline__ int stencil_cell_of(const RepConst& R, int t1, int t2, int t3,
                                               int nabor) {
  const int x = (map_off(nabor, 0) + t1 - 1 + R.ncells[0]) % R.ncells[0] + 1;
  const int y = (map_off(nabor, 1) + t2 - 1 + R.ncells[1]) % R.ncells[1] + 1;
  const int z = (map_off(nabor, 2) + t3 - 1 + R.ncells[2]) % R.ncells[2] + 1;
  return R.cell_off + (z * R.head_dim[1] + y) * R.head_dim[0] + x;
}

// Cell coordinates of a linear cell index of a replica.
__device__ __forceinline__ void cell_coords(const RepConst& R, int lin, int& x, int& y, int& z) {
  int l = lin - R.cell_off;
  x = l % R.head_dim[0];
  l /= R.head_dim[0];
  y = l % R.head_dim[1];
  z = l / R.head_dim[1];
}

// The stencil index (map order) of cell (a1, a2, a3) around the interior
// cell (t1, t2, t3), or -1: the wrapped offsets in {-1, 0, 1}^3 (at least 3
// cells along every axis, so that the 27 stencil cells are distinct).
__device__ __forceinline__ int stencil_index_of(const RepConst& R, int t1, int t2, int t3,
                                                int a1, int a2, int a3) {
  int o1 = a1 - t1, o2 = a2 - t2, o3 = a3 - t3;
  o1 = o1 > 1 ? o1 - R.ncells[0] : (o1 < -1 ? o1 + R.ncells[0] : o1);
  o2 = o2 > 1 ? o2 - R.ncells[1] : (o2 < -1 ? o2 + R.ncells[1] : o2);
  o3 = o3 > 1 ? o3 - R.ncells[2] : (o3 < -1 ? o3 + R.ncells[2] : o3);
  if (o1 < -1 || o1 > 1 || o2 < -1 || o2 > 1 || o3 < -1 || o3 > 1) return -1;
  return map_inv(o1, o2, o3);
}

__device__ __forceinline__ int stencil_cell(const RepConst& R, float4 Pf, const double4* P,
                                            int nabor) {
  int rc[3];
  cell_index3(R, Pf, P, rc[0], rc[1], rc[2]);
  int nc[3];
  for (int k = 0; k < 3; ++k) {
    int t = map_off(nabor, k) + rc[k] - 1;
    t = (t + R.ncells[k]) % R.ncells[k];
    nc[k] = t + 1;
  }
  return R.cell_off + (nc[2] * R.head_dim[1] + nc[1]) * R.head_dim[0] + nc[0];
}

// gcmc_run, one block of kGcmcThreads per replica.  With linked cells and no
// atom in a halo cell, the per-trial searches look only at the 27 cells
// around the trial point (cell edges >= rc + skin): the hard-core test over
// the gcmc group (`dr < rc^2` for some member, so the order of the search
// does not matter) and the appends to the lists of hs%ref members within
// rc + skin (each row gets at most one entry per insertion, so the order of
// the rows does not matter).  The m-th in-slab member of the deletion walk is
// found from per-chunk counts of in-slab members kept in shared memory
// (chunks of kGcmcThreads gorder positions), the first free slots from
// hints below which every slot is taken, and the group's first and last
// members (the template atom and the atom that receives the Maxwell
// velocity) are tracked across trials.  Replicas without cells, or with an
// atom in a halo cell, scan the whole group as the reference does.
__global__ void __launch_bounds__(kGcmcThreads) gcmc_kernel(Dev d, KParams p, int par) {
  DML_GRID_WAIT();
  if (par && d.grp[blockIdx.x].fast) return;  // decided by gcmc_fast_kernel
  if (threadIdx.x == 0) d.pr_cnt[blockIdx.x * kCntStride + kCntGcmcSeq] += 1;
  // dynamic shared memory: the trials, then in-slab members per gorder chunk
  extern __shared__ double4 s_dyn[];
  GcmcTrial* const s_tr = (GcmcTrial*)s_dyn;
  int* const s_chunk = (int*)(s_tr + kGcmcTrialBatch);
  const int rep = blockIdx.x;
  const RepConst& R = d.rc[rep];
  Scalars* const sc_g = d.sc + rep;
  // The replica's scalars live in shared memory for the whole call (one
  // thread updates them between barriers) and are written back at the end.
  __shared__ Scalars ss;
  Scalars* const sc = &ss;
  const int B = R.base;
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, wid = tid >> 5;
  const int nw = nt >> 5;
  __shared__ int s_first, s_last, s_n, s_slot, s_bslot, s_sel, s_dpre, s_pick, s_ppos;
  __shared__ int s_dec, s_m;
  __shared__ int s_cells[27], s_dup[27], s_start[27], s_pre[28], s_ca[27], s_cc[27];
  __shared__ int s_ccin[27], s_cbase[27];
  constexpr int KF = 8;  // flattened stencil entries a thread keeps in registers
  if (!sc_g->listed) {
    if (tid == 0) raise_error(d.g, DML_E_STATE, 0);
    return;
  }
  if (tid == 0) ss = *sc_g;
  __syncthreads();
  const long long step = d.g->step;
  const double z0 = sc->z0, zmax = sc->zmax;
  const double v = R.box[0] * R.box[1] * (zmax - z0);
  __shared__ int s_fast;
  // the trials' draws (the ran() calls of dana.F90:620-690, keyed Philox
  // here), kGcmcTrialBatch trials at a time
  auto draw_trials = [&](int t0) {
    __syncthreads();
    for (int i = tid; i < kGcmcTrialBatch && t0 + i <= p.nadj; i += nt) {
    const int t = t0 + i - 1;
    dml_u4 w0 = dml_draw(R.seed, step, (uint64_t)(t + 1), DML_RNG_GCMC, 0);
    dml_u4 w1 = dml_draw(R.seed, step, (uint64_t)(t + 1), DML_RNG_GCMC, 1);
    dml_u4 w2 = dml_draw(R.seed, step, (uint64_t)(t + 1), DML_RNG_GCMC, 2);
    GcmcTrial tr;
    tr.coin = dml_u53(w0.w[0], w0.w[1]);
    tr.uacc = dml_u53(w0.w[2], w0.w[3]);
    double r0 = dml_u53(w1.w[0], w1.w[1]) * R.box[0];
    double r1 = dml_u53(w1.w[2], w1.w[3]) * R.box[1];
    double r2 = dml_u53(w2.w[0], w2.w[1]) * (zmax - z0) + z0;
    tr.r = make_double4(r0, r1, r2, 0.0);
    tr.rf = make_float4((float)r0, (float)r1, (float)r2, 0.0f);
    tr.upick = dml_u53(w2.w[2], w2.w[3]);
    s_tr[i] = tr;
    }
  };
  if (R.use_cells)
    for (int c = tid; c < R.ncell; c += nt) d.ins_head[R.cell_off + c] = -1;
  // order arrays grow by appends: compact them before they could overflow
  if (sc->n_rank + p.nadj >= R.cap) {
    int n = blk_compact(d.ref, B, sc->n_rank, d.rank);
    if (tid == 0) sc->n_rank = n;
  }
  if (sc->n_alist + p.nadj >= R.cap) {
    int n = blk_compact(d.alist, B, sc->n_alist, d.apos);
    if (tid == 0) sc->n_alist = n;
  }
  if (sc->n_gorder + p.nadj >= R.cap) {
    int n = blk_compact(d.gorder, B, sc->n_gorder, d.gpos);
    if (tid == 0) sc->n_gorder = n;
  }
  __syncthreads();  // compacted counts visible to every thread
  if (tid == 0) {
    s_first = INT_MAX;
    s_last = -1;
    s_n = 0;
    s_fast = R.use_cells && !sc->halo;
  }
  {
    const int ng = sc->n_gorder;
    for (int k = tid; k * nt < ng; k += nt) s_chunk[k] = 0;
    __syncthreads();
    // in-slab count per chunk, the control-volume count n, first and last member
    int lo = INT_MAX, hi = -1;
    for (int base = 0; base < ng; base += nt) {
      int i = base + tid;
      int h = i < ng ? d.gorder[B + i] : -1;
      int in = 0;
      if (h >= 0) {
        lo = min(lo, i);
        hi = max(hi, i);
        in = in_slab(d.pos[h].z, z0, zmax);
      }
      unsigned m = __ballot_sync(0xffffffffu, in);
      if (lane == 0 && m) {
        atomicAdd(&s_chunk[base / nt], __popc(m));
        atomicAdd(&s_n, __popc(m));
      }
    }
    for (int off = 16; off > 0; off >>= 1) {
      lo = min(lo, __shfl_down_sync(0xffffffffu, lo, off));
      hi = max(hi, __shfl_down_sync(0xffffffffu, hi, off));
    }
    if (lane == 0) {
      atomicMin(&s_first, lo);
      atomicMax(&s_last, hi);
    }
  }
  for (int t = 1; t <= p.nadj; ++t) {
    if ((t - 1) % kGcmcTrialBatch == 0) draw_trials(t);
    __syncthreads();
    const GcmcTrial& tr = s_tr[(t - 1) % kGcmcTrialBatch];
    const int n = s_n, first = s_first, last = s_last;
    const bool fast = s_fast != 0;
    if (first == INT_MAX) {
      if (tid == 0) raise_error(d.g, DML_E_NO_PARTICLES, t);
      break;
    }
    const int ng = sc->n_gorder;
    // Metropolis decisions in one thread (FP64 on GB300's narrow pipe)
    if (tid == 0) {
      int dec;
      if (tr.coin < 0.5) {
        dec = (p.act * v / (double)(n + 1) < tr.uacc) ? 0 : 1;  // creation
      } else {
        dec = ((double)n / (v * p.act) < tr.uacc) ? 0 : 2;    // destruction
        int m = (int)floor(tr.upick * (double)n) + 1;
        s_m = m > n ? n : m;
      }
      s_dec = dec;
    }
    __syncthreads();
    const int dec = s_dec;
    if (dec == 0) continue;
    const int hlast = d.gorder[B + last];
    if (dec == 1) {
      // creation attempt (dana.F90:627-677)
      const int href = d.gorder[B + first];
      const double4 Rt = tr.r;
      const float4 Rtf = tr.rf;
      bool ov = false;
      // stencil entries (cell atoms) of this thread: slot, list flags, cell
      int fj[KF];
      int ff[KF], fq[KF];
      bool flat = false;
      if (fast) {
        if (tid < 27) {
          int c = stencil_cell(R, Rtf, &Rt, tid);
          int st = d.cell_start[c];
          s_cells[tid] = c;
          s_start[tid] = st;
          s_pre[tid] = d.cell_start[c + 1] - st;  // count, made a prefix below
          s_ca[tid] = 0;
        }
        __syncthreads();
        if (tid < 27) {
          int dup = 0;
          for (int q = 0; q < tid; ++q) dup |= s_cells[q] == s_cells[tid];
          s_dup[tid] = dup;
        }
        if (wid == 1) {
          int v = lane < 27 ? s_pre[lane] : 0, x = v;
          for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
          }
          if (lane < 27) s_pre[lane] = x - v;
          if (lane == 26) s_pre[27] = x;
        }
        __syncthreads();
        // The 27 cells as one index space f in [0, T): hard-core test over
        // the gcmc members among them, and (for the lists, if accepted) the
        // own-list and append flags from the same distance.
        const int T = s_pre[27];
        flat = T <= KF * nt;
#pragma unroll
        for (int k = 0; k < KF; ++k) {
          fj[k] = -1;
          ff[k] = 0;
          fq[k] = 0;
        }
        for (int k = 0, f = tid; f < T; ++k, f += nt) {
          int lo = 0, hi = 26;  // cell q with s_pre[q] <= f < s_pre[q + 1]
          while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (s_pre[mid] <= f) lo = mid; else hi = mid - 1;
          }
          const int q = lo;
          const int j = d.cell_atoms[s_start[q] + f - s_pre[q]];
          // FP32 distance decides outside the margins; FP64 (the
          // reference's vdistance, r - o%pos) inside them
          float fx, fy, fz;
          vdist_nint_f(R, Rtf, d.posf[j], fx, fy, fz);
          const float df = fx * fx + fy * fy + fz * fz;
          double rd = -1.0;
          auto exact = [&]() {
            if (rd < 0.0) {
              double vx, vy, vz;
              vdist_nint(R, Rt, d.pos[j], vx, vy, vz);
              rd = dot3(vx, vy, vz);
            }
            return rd;
          };
          if (df <= R.rc_hi2 && d.in_gcmc[j] && (df < R.rc_lo2 || exact() < p.rc2)) ov = true;
          if (flat && df <= R.rlist_hi2) {
            const bool live = d.state[j] == ST_LIVE;
            bool own, app;
            if (df < R.rlist_lo2) {
              own = app = true;
            } else {
              own = exact() < p.rlist2;
              app = !(exact() > p.rlist2);
            }
            int fl = 0;
            if (live && own) fl |= 1;  // own list (ngroup_cells_atom)
            if (live && app && !s_dup[q] && d.rank[j] >= 0) fl |= 2;  // append
#pragma unroll
            for (int kk = 0; kk < KF; ++kk)
              if (kk == k) {
                fj[kk] = j;
                ff[kk] = fl;
                fq[kk] = q;
              }
          }
        }
        if (tid < 27)  // this run's insertions, at the heads of the chains
          for (int h = d.ins_head[s_cells[tid]]; h >= 0 && !ov; h = d.ins_next[h]) {
            if (!d.in_gcmc[h]) continue;
            double vx, vy, vz;
            vdist_nint(R, Rt, d.pos[h], vx, vy, vz);
            if (dot3(vx, vy, vz) < p.rc2) ov = true;
          }
      } else {
        for (int i = tid; i < ng && !ov; i += nt) {
          int h = d.gorder[B + i];
          if (h < 0) continue;
          double vx, vy, vz;
          vdist_nint(R, Rt, d.pos[h], vx, vy, vz);
          if (dot3(vx, vy, vz) < p.rc2) ov = true;
        }
      }
      if (__syncthreads_or(ov)) continue;
      // first free hs slot (limbo slots are not free) and hs%b slot
      const int nat = sc->n_atoms + 1, bnat = sc->b_nat + 1;
      const int ns = sc->n_slots, nb = sc->n_b;
      {
        const int8_t* st = d.state + B;
        const int* b2 = d.b2hs + B;
        int res = ns >= nat + sc->nlimbo
                      ? blk_find_first(sc->free_lo, ns, [&](int i) { return st[i] == ST_NULL; },
                                       &s_slot)
                      : ns;
        int bres = nb >= bnat
                       ? blk_find_first(sc->bfree_lo, nb, [&](int b) { return b2[b] < 0; },
                                        &s_bslot)
                       : nb;
        if (tid == 0) {
          s_slot = res;
          s_bslot = bres;
        }
      }
      __syncthreads();
      const int lslot = s_slot, lbs = s_bslot;  // local hs and hs%b slots
      if (lslot == INT_MAX || lbs == INT_MAX) {
        if (tid == 0) raise_error(d.g, DML_E_INDEX, t);
        break;
      }
      if (lslot >= R.cap || lbs >= R.cap || sc->n_rank >= R.cap || sc->n_alist >= R.cap ||
          ng >= R.cap) {
        if (tid == 0) raise_error(d.g, DML_E_CAPACITY, t);
        break;
      }
      const int slot = B + lslot, bs = B + lbs;
      if (tid == 0) {
        // atom_asign(o, ref) then pos, pos_old = r (dana.F90:659-663); the
        // template's values are loaded before any store
        const int typ = d.typ[href];
        const double4 tv = d.vel[href], tf = d.force[href], ta = d.acel[href];
        const double te = d.epot[href];
        d.vel[slot] = tv;
        d.force[slot] = tf;
        if (p.mixed) atomicOr(&d.fnz[slot >> 5], 1u << (slot & 31));
        d.acel[slot] = ta;
        d.epot[slot] = te;
        d.typ[slot] = (int8_t)typ;
        d.pos[slot] = Rt;
        d.pos_old[slot] = Rt;
        d.posf_old[slot] = Rtf;
        d.old_cg[slot] = make_double4(1e8, 1e8, 1e8, 0.0);
        d.posf[slot] = to_f4(Rt, typ);
        d.skip[slot] = 0;
        d.id[slot] = sc->next_id;
        sc->next_id += 1;
        d.ev_count[slot] = 0;
        // Maxwell velocity to the last listed atom (dana.F90:666-668)
        const double beta = p.beta_t[typ - 1];
        double nv[4];
        dml_normal_quad(dml_draw(R.seed, step, (uint64_t)t, DML_RNG_GCMC_VEL, 0), nv);
        if (p.mixed)
          stv(d.vel, hlast, (float)(beta * nv[0]), (float)(beta * nv[1]), (float)(beta * nv[2]));
        else
          d.vel[hlast] = make_double4(beta * nv[0], beta * nv[1], beta * nv[2], 0.0);
        // sys
        int ap = sc->n_alist;
        d.alist[B + ap] = slot;
        d.apos[slot] = B + ap;
        sc->n_alist = ap + 1;
        // hs%ref
        int rk = sc->n_rank;
        d.ref[B + rk] = slot;
        d.rank[slot] = B + rk;
        sc->n_rank = rk + 1;
        sc->n_ref += 1;
        // hs%b (cgroup_attach_atom, Cells.F90:105-144)
        d.b2hs[bs] = slot;
        d.bslot[slot] = bs;
        if (lbs == nb) sc->n_b = nb + 1;
        sc->b_nat = bnat;
        sc->bfree_lo = lbs + 1;
        if (R.use_cells) {
          int c1, c2, c3;
          cell_index3(R, Rtf, &Rt, c1, c2, c3);
          if (c1 < 0 || c2 < 0 || c3 < 0 || c1 > R.ncells[0] + 1 || c2 > R.ncells[1] + 1 ||
              c3 > R.ncells[2] + 1) {
            raise_error(d.g, DML_E_OUT_OF_TESSELLATION, slot);
          } else {
            int c = R.cell_off + (c3 * R.head_dim[1] + c2) * R.head_dim[0] + c1;
            d.ins_next[slot] = d.ins_head[c];
            d.ins_head[c] = slot;
            // a halo cell is outside every stencil: full scans from here on
            if (c1 == 0 || c2 == 0 || c3 == 0 || c1 > R.ncells[0] || c2 > R.ncells[1] ||
                c3 > R.ncells[2])
              s_fast = 0;
          }
        }
        // hs (igroup slot)
        d.state[slot] = ST_LIVE;
        if (lslot == ns) sc->n_slots = ns + 1;
        sc->free_lo = lslot + 1;
        sc->n_atoms = nat;
        // gcmc: appended at the end of the group
        d.gorder[B + ng] = slot;
        d.gpos[slot] = B + ng;
        d.in_gcmc[slot] = 1;
        sc->n_gorder = ng + 1;
        sc->n_gcmc += 1;
        sc->gcmc_ins += 1;
        if (ng % nt == 0) s_chunk[ng / nt] = 0;  // a new chunk
        if (in_slab(Rt.z, z0, zmax)) s_chunk[ng / nt] += 1;
        s_last = ng;
        s_n = n + 1;
      }
      __syncthreads();
      // ngroup_sort_atom: own list, then append to every hs%ref list within reach
      auto append = [&](int j) {
        int m = d.nn[j];
        if (m >= p.mnb) {
          raise_error(d.g, DML_E_NEIGH_OVERFLOW, j);
          return;
        }
        d.list[(size_t)j * p.mnb + m] = slot;
        d.nn[j] = m + 1;
        flag_row(d, j);
      };
      if (flat) {
        // Own list in stencil order: per cell, this run's insertions (chain,
        // most recent first) then the sorted cell atoms in order.
#pragma unroll
        for (int k = 0; k < KF; ++k) {
          if (fj[k] < 0) continue;
          if (ff[k] & 1) atomicAdd(&s_ca[fq[k]], 1);
          if (ff[k] & 2) append(fj[k]);
        }
        if (tid < 27) {
          const int q = tid;
          int cnt = 0;
          for (int j = d.ins_head[s_cells[q]]; j >= 0; j = d.ins_next[j]) {
            if (j == slot || d.state[j] != ST_LIVE) continue;
            double vx, vy, vz;
            vdist_nint(R, d.pos[j], Rt, vx, vy, vz);
            double rd = dot3(vx, vy, vz);
            if (rd < p.rlist2) ++cnt;
            if (!s_dup[q] && d.rank[j] >= 0 && !(rd > p.rlist2)) append(j);
          }
          s_cc[q] = cnt;
        }
        __syncthreads();
        if (tid == 0) {
          int acc = 0, cc = 0;
          for (int q = 0; q < 27; ++q) {
            s_cbase[q] = acc;
            cc += s_cc[q];
            s_ccin[q] = cc;
            acc += s_cc[q] + s_ca[q];
          }
          if (acc > p.mnb) raise_error(d.g, DML_E_NEIGH_OVERFLOW, slot);
          d.nn[slot] = acc > p.mnb ? p.mnb : acc;
          list_new_row(d, slot);
        }
        __syncthreads();
        int* row = d.list + (size_t)slot * p.mnb;
        const int T = s_pre[27];
        int carry = 0;
#pragma unroll
        for (int k = 0; k < KF; ++k) {
          if (k * nt >= T) break;  // block-uniform
          int own = (fj[k] >= 0 && (ff[k] & 1)) ? 1 : 0;
          int tot;
          int e = blk_scan_excl(own, &tot);
          if (own) {
            int pos = s_ccin[fq[k]] + carry + e;
            if (pos < p.mnb) row[pos] = fj[k];
          }
          carry += tot;
        }
        if (tid < 27) {
          const int q = tid;
          int k = s_cbase[q];
          for (int j = d.ins_head[s_cells[q]]; j >= 0; j = d.ins_next[j]) {
            if (j == slot || d.state[j] != ST_LIVE) continue;
            double vx, vy, vz;
            vdist_nint(R, d.pos[j], Rt, vx, vy, vz);
            if (dot3(vx, vy, vz) < p.rlist2) {
              if (k < p.mnb) row[k] = j;
              ++k;
            }
          }
        }
      } else {
        if (wid == 0) gcmc_own_list(d, p, R, slot, sc->n_b);
        if (fast) {
          for (int q = wid; q < 27; q += nw) {
            if (s_dup[q]) continue;
            int c = s_cells[q];
            int start = d.cell_start[c], num = d.cell_start[c + 1] - start;
            for (int idx = lane; idx < num; idx += 32) {
              int j = d.cell_atoms[start + idx];
              if (j == slot || d.state[j] != ST_LIVE || d.rank[j] < 0) continue;
              if (list_entry_in(p, R, Rt, d.pos[j], false)) append(j);
            }
            if (lane == 0)
              for (int j = d.ins_head[c]; j >= 0; j = d.ins_next[j]) {
                if (j == slot || d.state[j] != ST_LIVE || d.rank[j] < 0) continue;
                if (list_entry_in(p, R, Rt, d.pos[j], false)) append(j);
              }
          }
        } else {
          int nr = sc->n_rank;
          for (int q = tid; q < nr; q += nt) {
            int j = d.ref[B + q];
            if (j < 0 || j == slot) continue;
            if (list_entry_in(p, R, Rt, d.pos[j], false)) append(j);
          }
        }
      }
    } else {
      // destruction attempt (dana.F90:680-707)
      const int m = s_m;
      int hsel = -1, psel = -1;
      if (m <= 0) {
        hsel = hlast;  // the walk never reaches m == 0 and ends on the last atom
        psel = last;
      } else {
        // chunk holding the m-th in-slab member
        if (tid == 0) {
          s_sel = -1;
          s_pick = -1;
        }
        const int nch = (ng + nt - 1) / nt;
        int carry = 0;
        for (int base = 0; base < nch; base += nt) {
          int k = base + tid;
          int c = k < nch ? s_chunk[k] : 0;
          int tot;
          int pre = blk_scan_excl(c, &tot);
          if (c > 0 && carry + pre < m && m <= carry + pre + c) {
            s_sel = k;
            s_dpre = carry + pre;
          }
          carry += tot;
          if (carry >= m) break;
        }
        __syncthreads();
        const int k = s_sel;
        if (k < 0) {
          if (tid == 0) raise_error(d.g, DML_E_CHOSEN_MISSING, t);
          break;
        }
        int i = k * nt + tid;
        int h = i < ng ? d.gorder[B + i] : -1;
        bool in = h >= 0 && in_slab(d.pos[h].z, z0, zmax);
        int tot;
        int pre = blk_scan_excl(in ? 1 : 0, &tot);
        if (in && s_dpre + pre + 1 == m) {
          s_pick = h;
          s_ppos = i;
        }
        __syncthreads();
        hsel = s_pick;
        psel = s_ppos;
        if (hsel < 0) {
          if (tid == 0) raise_error(d.g, DML_E_CHOSEN_MISSING, t);
          break;
        }
      }
      if (tid == 0) {
        // atom_destroy: gcmc, hs (nn, hs%ref, hs%b), sys (Groups.F90:433-467);
        // the atom's indices are loaded before any store
        const int h = hsel;
        const double4 P = d.pos[h];
        const int gp = d.gpos[h], rk = d.rank[h], bsl = d.bslot[h], ap = d.apos[h];
        const float4 pf = d.posf[h];
        if (in_slab(P.z, z0, zmax)) s_chunk[psel / nt] -= 1;
        d.in_gcmc[h] = 0;
        d.gorder[gp] = -1;
        sc->n_gcmc -= 1;
        d.nn[h] = 0;
        if (rk >= 0) {
          d.ref[rk] = -1;
          d.rank[h] = -1;
          sc->n_ref -= 1;
        }
        if (R.use_cells) {
          int c1, c2, c3;
          cell_index3(R, pf, &P, c1, c2, c3);
          if (c1 < 0 || c2 < 0 || c3 < 0 || c1 > R.ncells[0] || c2 > R.ncells[1] || c3 > R.ncells[2])
            raise_error(d.g, DML_E_UNSUPPORTED, h);  // tessellation dropped (Cells.F90:320-327)
        }
        d.b2hs[bsl] = -1;
        d.bslot[h] = -1;
        if (bsl - B < sc->bfree_lo) sc->bfree_lo = bsl - B;
        sc->b_nat -= 1;
        d.state[h] = ST_LIMBO;
        sc->nlimbo += 1;
        sc->n_atoms -= 1;
        d.posf[h] = make_float4(pf.x, pf.y, pf.z, __int_as_float(0));
        d.alist[ap] = -1;
        sc->gcmc_del += 1;
        s_n = n - 1;
      }
      __syncthreads();
      // new first / last member when one of them left the group
      if (wid == 0 && psel == first) {
        int res = INT_MAX;
        for (int base = psel + 1; base < ng; base += 32) {
          int i = base + lane;
          unsigned mk = __ballot_sync(0xffffffffu, i < ng && d.gorder[B + i] >= 0);
          if (mk) {
            res = base + __ffs(mk) - 1;
            break;
          }
        }
        if (lane == 0) s_first = res;
      }
      if (wid == 1 && psel == last) {
        int res = -1;
        for (int top = psel - 1; top >= 0; top -= 32) {
          int i = top - lane;
          unsigned mk = __ballot_sync(0xffffffffu, i >= 0 && d.gorder[B + i] >= 0);
          if (mk) {
            res = top - (__ffs(mk) - 1);
            break;
          }
        }
        if (lane == 0) s_last = res;
      }
    }
  }
  __syncthreads();
  if (tid == 0) {
    ss.halo = 0;
    *sc_g = ss;
  }
}

// ------------------------------------------- gcmc_run with linked cells
// The trials of gcmc_run are sequential, but on a replica with linked cells
// whose atoms and trial points all lie in interior cells, everything a trial
// reads can be found before any trial is decided:
//  * its uniforms and point (keyed draws);
//  * the gcmc members within rc of its point at the start of the call (the
//    hard-core "blockers", recorded by gcmc%alist position): a member blocks
//    the trial unless an earlier trial deleted it;
//  * the earlier trial points within rc (an earlier insertion blocks it);
//  * the atoms within rc + skin among its 27 stencil cells (own list and
//    appends), each used unless deleted before the trial;
//  * the membership and in-slab bits of every gcmc%alist position (the m-th
//    in-slab member of a deletion);
//  * the free hs and hs%b slots (igroup_attach_atom takes the first one).
// gcmc_pre_kernel finds all of it, one block per replica; gcmc_fast_kernel
// then decides the trials in order in one warp on shared-memory state and
// applies their edits with the whole block.  A replica that does not
// qualify (no cells, an atom or point in a halo cell, more than
// kGcmcMaxTrials trials, a point with more than kGcmcBlk blockers or
// kGcmcCand list atoms) runs gcmc_kernel instead.
constexpr int kGcmcPreThreads = 512;
constexpr int kGcmcPairQ = 2048;  // queued pairs within rc + skin (more: sequential path)

__device__ __forceinline__ bool hard_core_in(const KParams& p, const RepConst& R, double4 a,
                                             float4 af, double4 b, float4 bf) {
  // |a - b|^2 < rc^2 (dana.F90:649-651), FP32 outside the margins
  float fx, fy, fz;
  vdist_nint_f(R, af, bf, fx, fy, fz);
  const float df = fx * fx + fy * fy + fz * fz;
  if (df > R.rc_hi2) return false;
  if (df < R.rc_lo2) return true;
  double vx, vy, vz;
  vdist_nint(R, a, b, vx, vy, vz);
  return dot3(vx, vy, vz) < p.rc2;
}

// First `want` positions q in [lo, hi) with free(q), ascending, into out[];
// returns how many were found.  Every thread of the block calls it; per
// round each thread tests a run of kCollectV consecutive positions (their
// loads all in flight), one block scan places the finds.
constexpr int kCollectV = 32;
template <class Pred>
__device__ int blk_collect(int lo, int hi, int want, Pred free_at, int* out, int* s_cnt) {
  if (threadIdx.x == 0) *s_cnt = 0;
  __syncthreads();
  for (int base = lo; base < hi; base += kCollectV * (int)blockDim.x) {
    const int q0 = base + kCollectV * (int)threadIdx.x;
    unsigned m = 0u;
#pragma unroll
    for (int v = 0; v < kCollectV; ++v)
      if (q0 + v < hi && free_at(q0 + v)) m |= 1u << v;
    int tot;
    const int pre = blk_scan_excl(__popc(m), &tot);
    int k = *s_cnt + pre;
    while (m != 0u && k < want) {
      out[k++] = q0 + __ffs(m) - 1;
      m &= m - 1u;
    }
    __syncthreads();
    if (threadIdx.x == 0) *s_cnt += tot;
    __syncthreads();
    if (*s_cnt >= want) break;
  }
  const int n = min(*s_cnt, want);
  __syncthreads();
  return n;
}

__global__ void __launch_bounds__(kGcmcPreThreads) gcmc_pre_kernel(Dev d, KParams p) {
  DML_GRID_WAIT();
  const int rep = blockIdx.x;
  const RepConst& R = d.rc[rep];
  Scalars* const sc = d.sc + rep;
  GcmcRepPre* const gr = d.grp + rep;
  const int B = R.base, tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, wid = tid >> 5;
  const int nw = nt >> 5;
  const unsigned lt = (1u << lane) - 1u;
  __shared__ int s_bad, s_cnt, s_ncrt;
  __shared__ double4 s_r[kGcmcMaxTrials];
  __shared__ float4 s_rf[kGcmcMaxTrials];
  __shared__ unsigned char s_crt[kGcmcMaxTrials];
  // per creation trial (compacted): trial, cell, repeats, row segments of
  // its stencil in gs (start, exclusive prefix of the sizes), counts
  __shared__ int s_nct;
  __shared__ short s_ct[kGcmcMaxTrials];
  __shared__ short s_tc[kGcmcMaxTrials][3];  // by trial: the point's cell
  __shared__ unsigned s_dup[kGcmcMaxTrials];
  __shared__ int s_segst[kGcmcMaxTrials][9], s_segpre[kGcmcMaxTrials][10];
  __shared__ int s_tpre[kGcmcMaxTrials + 1];
  __shared__ int s_nb[kGcmcMaxTrials], s_nc[kGcmcMaxTrials];
  __shared__ unsigned s_pm[kGcmcMaxTrials][kGcmcMaskW];
  __shared__ int s_npq;                  // pairs within rc + skin: (trial, place in gs)
  __shared__ int2 s_pq[kGcmcPairQ];
  extern __shared__ int rowend[];  // the row ends of the cell-row sort
  if (!sc->listed) {  // gcmc_kernel reports the state error
    if (tid == 0) gr->fast = 0;
    return;
  }
  const int nrows = R.head_dim[1] * R.head_dim[2];
  const int n_gl = d.pr_cnt[rep * kCntStride + kCntGlist];
  if (tid == 0) {
    s_bad = !(R.use_cells && !sc->halo && p.nadj <= kGcmcMaxTrials && nrows <= d.gcmc_rows);
    s_ncrt = 0;
    s_nct = 0;
    s_npq = 0;
  }
  __syncthreads();
  if (s_bad) {
    if (tid == 0) gr->fast = 0;
    return;
  }
  const long long step = d.g->step;
  const double z0 = sc->z0, zmax = sc->zmax;
  GcmcTrialPre* const pre = d.gpre + (size_t)rep * kGcmcMaxTrials;
  unsigned* const pm = d.gpm + (size_t)rep * kGcmcMaxTrials * kGcmcMaskW;

  // The trials' draws (dana.F90:620-690, keyed Philox) and points.
  if (tid < p.nadj) {
    const int t = tid + 1;
    GcmcTrialPre& tr = pre[tid];
    dml_u4 w0 = dml_draw(R.seed, step, (uint64_t)t, DML_RNG_GCMC, 0);
    dml_u4 w1 = dml_draw(R.seed, step, (uint64_t)t, DML_RNG_GCMC, 1);
    dml_u4 w2 = dml_draw(R.seed, step, (uint64_t)t, DML_RNG_GCMC, 2);
    const double coin = dml_u53(w0.w[0], w0.w[1]);
    const double r0 = dml_u53(w1.w[0], w1.w[1]) * R.box[0];
    const double r1 = dml_u53(w1.w[2], w1.w[3]) * R.box[1];
    const double r2 = dml_u53(w2.w[0], w2.w[1]) * (zmax - z0) + z0;
    const double4 r = make_double4(r0, r1, r2, 0.0);
    const float4 rf = to_f4(r, 0);
    tr.r = r;
    tr.coin = coin;
    tr.uacc = dml_u53(w0.w[2], w0.w[3]);
    tr.upick = dml_u53(w2.w[2], w2.w[3]);
    tr.kpick = ((unsigned long long)(w2.w[2] >> 5) << 26) | (w2.w[3] >> 6);
    const bool crt = coin < 0.5;
    s_r[tid] = r;
    s_rf[tid] = rf;
    s_crt[tid] = crt;
    tr.n_blk = 0;
    tr.n_cand = 0;
    if (crt) {
      atomicAdd(&s_ncrt, 1);
      double nv[4];
      dml_normal_quad(dml_draw(R.seed, step, (uint64_t)t, DML_RNG_GCMC_VEL, 0), nv);
      tr.nv[0] = nv[0];
      tr.nv[1] = nv[1];
      tr.nv[2] = nv[2];
      int c1, c2, c3;
      cell_index3(R, rf, &r, c1, c2, c3);
      // a point outside the interior cells (or the tessellation) takes the
      // sequential path, which reports or handles it as the reference does
      if (c1 < 1 || c2 < 1 || c3 < 1 || c1 > R.ncells[0] || c2 > R.ncells[1] || c3 > R.ncells[2])
        s_bad = 1;
      tr.cell = R.cell_off + (c3 * R.head_dim[1] + c2) * R.head_dim[0] + c1;
      s_tc[tid][0] = (short)c1;
      s_tc[tid][1] = (short)c2;
      s_tc[tid][2] = (short)c3;
      s_ct[atomicAdd(&s_nct, 1)] = (short)tid;
    }
  }
  for (int e = tid; e < kGcmcMaxTrials * kGcmcMaskW; e += nt) (&s_pm[0][0])[e] = 0u;
  // The atoms gcmc_bin_kernel listed (live, in the layers the trials reach),
  // counting-sorted by cell row (z layer, y row), the counts in shared
  // memory: row r's FP32 positions and hs slots are gs[rowend[r - 1] ..
  // rowend[r]) (from 0 for r = 0), contiguous for the searches below.
  const int hd0 = R.head_dim[0];
  for (int r = tid; r < nrows; r += nt) rowend[r] = 0;
  __syncthreads();
  const int2* const gl = d.glist + B;
  constexpr int kSortU = 4;  // entries per thread per round, loads in flight together
  for (int i0 = tid; i0 < n_gl; i0 += kSortU * nt) {
    int cl[kSortU];
#pragma unroll
    for (int u = 0; u < kSortU; ++u) cl[u] = i0 + u * nt < n_gl ? gl[i0 + u * nt].y : -1;
#pragma unroll
    for (int u = 0; u < kSortU; ++u)
      if (cl[u] >= 0) atomicAdd(&rowend[(cl[u] - R.cell_off) / hd0], 1);
  }
  __syncthreads();
  {
    const int per = (nrows + nt - 1) / nt, r0 = tid * per, r1 = min(r0 + per, nrows);
    int sum = 0;
    for (int r = r0; r < r1; ++r) sum += rowend[r];
    int tot;
    int run = blk_scan_excl(sum, &tot);
    for (int r = r0; r < r1; ++r) {
      const int c = rowend[r];
      rowend[r] = run;  // the row's start, advanced to its end by the scatter
      run += c;
    }
  }
  __syncthreads();
  float4* const gs = d.gsort + B;
  for (int i0 = tid; i0 < n_gl; i0 += kSortU * nt) {
    int cl[kSortU];
    float4 rec[kSortU];
#pragma unroll
    for (int u = 0; u < kSortU; ++u) {
      const bool on = i0 + u * nt < n_gl;
      cl[u] = on ? gl[i0 + u * nt].y : -1;
      rec[u] = on ? d.glp[B + i0 + u * nt] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int u = 0; u < kSortU; ++u)
      if (cl[u] >= 0) gs[atomicAdd(&rowend[(cl[u] - R.cell_off) / hd0], 1)] = rec[u];
  }
  __syncthreads();

  // Earlier creation points within rc of each creation point: an accepted
  // earlier insertion sits there during this trial's hard-core test (all
  // ordered pairs of creation trials of the block).
  const int nct = s_nct;
  for (int e = tid; e < nct * nct; e += nt) {
    const int ia = s_ct[e / nct], ib = s_ct[e % nct];
    if (ib < ia && hard_core_in(p, R, s_r[ia], s_rf[ia], s_r[ib], s_rf[ib]))
      atomicOr(&s_pm[ia][ib >> 5], 1u << (ib & 31));
  }
  __syncthreads();
  for (int e = tid; e < p.nadj * kGcmcMaskW; e += nt) pm[e] = (&s_pm[0][0])[e];

  // Blockers and list candidates of every creation trial: the atoms of the
  // (at most 9) cell rows through its 27 stencil cells within rc + skin
  // (FP32, FP64 inside the margins), each matched to the stencil cells that
  // hold it; the candidates then put in the order of the stencil walk (map
  // order, each cell by descending hs%b slot).  Setup per creation trial,
  // then all (trial, row atom) pairs of the block, then a sort per trial.
  const int n1 = R.ncells[0], n2 = R.ncells[1], n3 = R.ncells[2];
  const int hd1 = R.head_dim[1];
  // fewer than 3 cells along an axis: stencil cells repeat
  const bool small = n1 < 3 || n2 < 3 || n3 < 3;
  // the stencil cells (map order) of every creation trial
  for (int e = tid; e < nct * 27; e += nt) {
    const int i = s_ct[e / 27], q = e % 27;
    pre[i].cells[q] = stencil_cell_of(R, s_tc[i][0], s_tc[i][1], s_tc[i][2], q);
  }
  // the 9 rows (dz, dy) through the stencil: start in gs, size
  for (int e = tid; e < nct * 9; e += nt) {
    const int c = e / 9, k = e % 9, i = s_ct[c];
    const int z = (s_tc[i][2] - 1 + k / 3 - 1 + n3) % n3 + 1;
    const int y = (s_tc[i][1] - 1 + k % 3 - 1 + n2) % n2 + 1;
    const int row = z * hd1 + y;
    const int st = row > 0 ? rowend[row - 1] : 0;
    s_segst[c][k] = st;
    s_segpre[c][k] = rowend[row] - st;  // the size; a prefix below
  }
  __syncthreads();
  for (int c = tid; c < nct; c += nt) {
    const int i = s_ct[c];
    unsigned dupm = 0u;
    if (small) {
      // a repeated stencil cell (dup bit), a repeated row (scanned once)
      for (int q = 1; q < 27; ++q)
        for (int q2 = 0; q2 < q; ++q2)
          if (pre[i].cells[q2] == pre[i].cells[q]) {
            dupm |= 1u << q;
            break;
          }
      for (int k = 1; k < 9; ++k)
        for (int k2 = 0; k2 < k; ++k2)
          if ((s_tc[i][2] - 1 + k / 3 - 1 + n3) % n3 == (s_tc[i][2] - 1 + k2 / 3 - 1 + n3) % n3 &&
              (s_tc[i][1] - 1 + k % 3 - 1 + n2) % n2 == (s_tc[i][1] - 1 + k2 % 3 - 1 + n2) % n2) {
            s_segpre[c][k] = 0;
            break;
          }
    }
    int T = 0;
    for (int k = 0; k < 9; ++k) {
      const int sz = s_segpre[c][k];
      s_segpre[c][k] = T;
      T += sz;
    }
    s_segpre[c][9] = T;
    s_tpre[c] = T;
    s_dup[c] = dupm;
    s_nb[c] = 0;
    s_nc[c] = 0;
  }
  __syncthreads();
  // the pairs of each creation trial start at the exclusive prefix s_tpre
  {
    const int v = tid < nct ? s_tpre[tid] : 0;
    int tot;
    const int e = blk_scan_excl(v, &tot);
    if (tid < nct) s_tpre[tid] = e;
    if (tid == 0) s_tpre[nct] = tot;
  }
  __syncthreads();
  // Every (trial, row atom) pair of the block: each thread walks a
  // contiguous range of them (so a row's records are read in order), kPairU
  // loads in flight; the pairs within rc + skin (FP32 with margin) are queued
  // and then evaluated by the whole block.
  constexpr int kPairU = 4;
  const int npair = s_tpre[nct];
  {
    const int per = (npair + nt - 1) / nt;
    const int e_beg = min(tid * per, npair), e_end = min(e_beg + per, npair);
    int c = 0, k = 0;
    if (e_beg < e_end) {
      int lo = 0, hi = nct - 1;  // the trial: last c with s_tpre[c] <= e_beg
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (s_tpre[mid] <= e_beg) lo = mid; else hi = mid - 1;
      }
      c = lo;
      while (s_segpre[c][k + 1] <= e_beg - s_tpre[c]) ++k;
    }
    for (int e = e_beg; e < e_end;) {
      const int f = e - s_tpre[c];
      const int len = min(s_segpre[c][k + 1] - f, e_end - e);
      const int g0 = s_segst[c][k] + f - s_segpre[c][k];
      const float4 Rtf = s_rf[s_ct[c]];
      for (int r0 = 0; r0 < len; r0 += kPairU) {
        float4 QQ[kPairU];
#pragma unroll
        for (int u = 0; u < kPairU; ++u)
          QQ[u] = r0 + u < len ? gs[g0 + r0 + u] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int u = 0; u < kPairU; ++u) {
          float fx, fy, fz;
          vdist_nint_f(R, Rtf, QQ[u], fx, fy, fz);
          const float df = fx * fx + fy * fy + fz * fz;
          if (r0 + u < len && df <= R.rlist_hi2) {
            const int qn = atomicAdd(&s_npq, 1);
            if (qn < kGcmcPairQ) s_pq[qn] = make_int2(c, g0 + r0 + u);
          }
        }
      }
      e += len;
      if (e < e_end) {  // the next segment with pairs (of this trial or a later one)
        while (s_tpre[c + 1] <= e) ++c, k = 0;
        const int f2 = e - s_tpre[c];
        while (s_segpre[c][k + 1] <= f2) ++k;
      }
    }
  }
  __syncthreads();
  if (tid == 0 && s_npq > kGcmcPairQ) s_bad = 1;
  const int npq = min(s_npq, kGcmcPairQ);
  for (int x = tid; x < npq; x += nt) {
    const int c = s_pq[x].x, i = s_ct[c];
    const float4 Q = gs[s_pq[x].y];
    const int j = __float_as_int(Q.w);
    float fx, fy, fz;
    vdist_nint_f(R, s_rf[i], Q, fx, fy, fz);
    const float df = fx * fx + fy * fy + fz * fz;
    int a1, a2, a3;
    cell_index3(R, Q, d.pos + j, a1, a2, a3);  // its cell in the cell sort
    const bool mem = d.in_gcmc[j] != 0;
    const bool inref = d.rank[j] >= 0;
    const unsigned key = ~(unsigned)d.bslot[j];
    double rd = -1.0;  // FP64 only inside the margins of rc and rc + skin
    if (df >= R.rlist_lo2 || (mem && df >= R.rc_lo2 && df <= R.rc_hi2)) {
      double vx, vy, vz;
      vdist_nint(R, s_r[i], d.pos[j], vx, vy, vz);
      rd = dot3(vx, vy, vz);
    }
    const bool isb = df <= R.rc_hi2 && mem && (df < R.rc_lo2 || rd < p.rc2);
    const bool own = df < R.rlist_lo2 || rd < p.rlist2;
    const bool app = (df < R.rlist_lo2 || !(rd > p.rlist2)) && inref;
    GcmcTrialPre& tr = pre[i];
    const unsigned dupm = s_dup[c];
    auto emit = [&](int q) {
      if (isb) {
        const int kb = atomicAdd(&s_nb[c], 1);
        if (kb < kGcmcBlk) tr.blk[kb] = d.gpos[j] - B;
      }
      const int fl = (own ? 1 : 0) | (app && !((dupm >> q) & 1u) ? 2 : 0);
      if (fl) {
        const int kc = atomicAdd(&s_nc[c], 1);
        if (kc < kGcmcCand) {
          tr.cand[kc] = j;
          tr.cq[kc] = (unsigned char)q;
          tr.cf[kc] = (unsigned char)fl;
          tr.ckey[kc] = key;
        }
      }
    };
    if (!small) {
      // the offset from the trial's cell, wrapped; a stencil cell when in {-1, 0, 1}^3
      int o1 = a1 - s_tc[i][0], o2 = a2 - s_tc[i][1], o3 = a3 - s_tc[i][2];
      o1 = o1 > 1 ? o1 - n1 : (o1 < -1 ? o1 + n1 : o1);
      o2 = o2 > 1 ? o2 - n2 : (o2 < -1 ? o2 + n2 : o2);
      o3 = o3 > 1 ? o3 - n3 : (o3 < -1 ? o3 + n3 : o3);
      if (o1 >= -1 && o1 <= 1 && o2 >= -1 && o2 <= 1 && o3 >= -1 && o3 <= 1)
        emit(map_inv(o1, o2, o3));
    } else {
      const int lin = R.cell_off + (a3 * hd1 + a2) * R.head_dim[0] + a1;
      for (int q = 0; q < 27; ++q)
        if (tr.cells[q] == lin) emit(q);
    }
  }
  __syncthreads();
  // each trial's candidates in stencil-walk order (a rank sort per warp)
  for (int c = wid; c < nct; c += nw) {
    GcmcTrialPre& tr = pre[s_ct[c]];
    const int nb = s_nb[c], nc = s_nc[c], nk = min(nc, kGcmcCand);
    int j0 = -1, j1 = -1, q0 = 0, q1 = 0, f0 = 0, f1 = 0;
    unsigned long long k0 = ~0ull, k1 = ~0ull;
    if (lane < nk) {
      j0 = tr.cand[lane];
      q0 = tr.cq[lane];
      f0 = tr.cf[lane];
      k0 = ((unsigned long long)q0 << 32) | tr.ckey[lane];
    }
    if (lane + 32 < nk) {
      j1 = tr.cand[lane + 32];
      q1 = tr.cq[lane + 32];
      f1 = tr.cf[lane + 32];
      k1 = ((unsigned long long)q1 << 32) | tr.ckey[lane + 32];
    }
    int r0 = 0, r1 = 0;
    for (int m = 0; m < nk; ++m) {
      const unsigned long long km = __shfl_sync(0xffffffffu, m < 32 ? k0 : k1, m & 31);
      r0 += km < k0;
      r1 += km < k1;
    }
    __syncwarp();
    if (lane < nk) {
      tr.cand[r0] = j0;
      tr.cq[r0] = (unsigned char)q0;
      tr.cf[r0] = (unsigned char)f0;
    }
    if (lane + 32 < nk) {
      tr.cand[r1] = j1;
      tr.cq[r1] = (unsigned char)q1;
      tr.cf[r1] = (unsigned char)f1;
    }
    if (lane == 0) {
      tr.n_blk = nb;
      tr.n_cand = nc;
      tr.dup = s_dup[c];
      if (nb > kGcmcBlk || nc > kGcmcCand) s_bad = 1;
    }
  }
  __syncthreads();

  // The first free hs and hs%b slots (igroup_attach_atom, Groups.F90:
  // 1083-1093): every insertion takes the lowest, deletions free no hs slot
  // (limbo) but free their hs%b slot at once.
  const int ncrt = s_ncrt;
  const int ns = sc->n_slots, nbs = sc->n_b;
  const int holes = ns - sc->n_atoms - sc->nlimbo;
  const int bholes = nbs - sc->b_nat;
  const int8_t* st = d.state + B;
  const int* b2 = d.b2hs + B;
  int nh = 0, nbh = 0;
  if (holes > 0 && ncrt > 0)
    nh = blk_collect(sc->free_lo, ns, min(holes, ncrt), [&](int q) { return st[q] == ST_NULL; },
                     gr->holes, &s_cnt);
  if (bholes > 0 && ncrt > 0)
    nbh = blk_collect(sc->bfree_lo, nbs, min(bholes, ncrt), [&](int q) { return b2[q] < 0; },
                      gr->bholes, &s_cnt);
  if (tid == 0) {
    gr->n_holes = nh;
    gr->n_bholes = nbh;
    gr->fast = !s_bad;
  }
}

constexpr int kGcmcFastThreads = 512;
constexpr int kGcmcAppCap = 768;  // appends kept in shared memory (else applied trial by trial)

struct Vel3 {
  double x, y, z;
};

// Shared state of gcmc_fast_kernel (dynamic shared memory, followed by the
// in-slab counts per 1024 positions and, when they fit, the bit words).
struct GcmcSm {
  Scalars ss;
  double uacc[kGcmcMaxTrials];
  unsigned long long kpick[kGcmcMaxTrials];
  unsigned char crt[kGcmcMaxTrials], rin[kGcmcMaxTrials];  // creation trial; point in the slab
  int nblk[kGcmcMaxTrials];
  int blk[kGcmcMaxTrials][kGcmcBlk];
  unsigned pm[kGcmcMaxTrials][kGcmcMaskW];
  unsigned acc[kGcmcMaskW];  // trials whose insertion is a member now
  int holes[kGcmcMaxTrials], bholes[kGcmcMaxTrials];
  int nholes, nbholes;
  // accepted insertions, in trial order (local slots)
  int ins_trial[kGcmcMaxTrials], ins_slot[kGcmcMaxTrials], ins_bslot[kGcmcMaxTrials];
  int ins_fpos[kGcmcMaxTrials], ins_lpos[kGcmcMaxTrials], ins_gpos[kGcmcMaxTrials];
  int ins_rank[kGcmcMaxTrials], ins_alist[kGcmcMaxTrials], ins_cell[kGcmcMaxTrials];
  int ins_del[kGcmcMaxTrials];  // trial that deleted the inserted atom, or INT_MAX
  long long ins_id[kGcmcMaxTrials];
  int pos2ins[kGcmcMaxTrials];  // insertion at gcmc%alist position ng0 + x
  // accepted deletions, in trial order
  int del_trial[kGcmcMaxTrials], del_pos[kGcmcMaxTrials], del_slot[kGcmcMaxTrials];
  int del_bslot[kGcmcMaxTrials], del_reused[kGcmcMaxTrials], del_kins[kGcmcMaxTrials];
  int freed[kGcmcMaxTrials], freed_del[kGcmcMaxTrials];  // min-heap of freed hs%b slots
  double qc[2 * kGcmcMaxTrials + 1], qd[2 * kGcmcMaxTrials + 1];  // acceptance quotients
  int nins, ndel;
  // edits
  int href[kGcmcMaxTrials], hlast[kGcmcMaxTrials], href_ins[kGcmcMaxTrials];
  int hlast_ins[kGcmcMaxTrials], root[kGcmcMaxTrials], htyp[kGcmcMaxTrials], ityp[kGcmcMaxTrials];
  Vel3 tvel[kGcmcMaxTrials], fvel[kGcmcMaxTrials];
  float4 nv[kGcmcMaxTrials];  // Maxwell normals (FP32 values, exact)
  int mw_slot[kGcmcMaxTrials];
  Vel3 mw_vel[kGcmcMaxTrials];
  int n_mw;
  int napp, app_over;
  int app_j[kGcmcAppCap], app_k[kGcmcAppCap], app_base[kGcmcAppCap];
};

// The m-th (1-based) set bit of the in-slab words over positions [0, ng),
// or -1; one warp.
__device__ int warp_select(const unsigned* wsl, const int* grp, int ng, int m) {
  const int lane = threadIdx.x & 31;
  const int ngrp = (ng + 1023) >> 10;
  int acc = 0;
  for (int g0 = 0; g0 < ngrp; g0 += 32) {
    const int g = g0 + lane;
    const int c = g < ngrp ? grp[g] : 0;
    int x = c;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    const unsigned hit = __ballot_sync(0xffffffffu, acc + x >= m);
    if (hit) {
      const int L = __ffs(hit) - 1;
      const int gg = g0 + L;
      const int mr = m - acc - __shfl_sync(0xffffffffu, x - c, L);
      const int wi = gg * 32 + lane;
      const unsigned w = wi * 32 < ng ? wsl[wi] : 0u;
      const int wc = __popc(w);
      int y = wc;
      for (int o = 1; o < 32; o <<= 1) {
        const int z = __shfl_up_sync(0xffffffffu, y, o);
        if (lane >= o) y += z;
      }
      const unsigned hit2 = __ballot_sync(0xffffffffu, y >= mr);
      if (!hit2) return -1;
      const int L2 = __ffs(hit2) - 1;
      const int k = mr - __shfl_sync(0xffffffffu, y - wc, L2);
      const unsigned ww = __shfl_sync(0xffffffffu, w, L2);
      const bool set = (ww >> lane) & 1u;
      const int below = __popc(ww & ((1u << lane) - 1u));
      const unsigned hit3 = __ballot_sync(0xffffffffu, set && below == k - 1);
      if (!hit3) return -1;
      return (gg * 32 + L2) * 32 + (__ffs(hit3) - 1);
    }
    acc += __shfl_sync(0xffffffffu, x, 31);
  }
  return -1;
}

// warp_select with the inclusive in-slab counts per 1024 positions held in
// registers (group lane in P0, group lane + 32 in P1): the group is one
// ballot, the word a scan of its 32 words, the bit a ballot.
__device__ int warp_select_reg(const unsigned* wsl, int P0, int P1, int ng, int m) {
  const int lane = threadIdx.x & 31;
  const unsigned h0 = __ballot_sync(0xffffffffu, P0 >= m), h1 = __ballot_sync(0xffffffffu, P1 >= m);
  if (!h0 && !h1) return -1;
  const int gg = h0 ? __ffs(h0) - 1 : 32 + __ffs(h1) - 1;
  const int gp = gg - 1;  // members before group gg
  const int before0 = __shfl_sync(0xffffffffu, P0, gp & 31), before1 = __shfl_sync(0xffffffffu, P1, gp & 31);
  const int mr = m - (gp < 0 ? 0 : (gp < 32 ? before0 : before1));
  const int wi = gg * 32 + lane;
  const unsigned w = wi * 32 < ng ? wsl[wi] : 0u;
  const int wc = __popc(w);
  int y = wc;
  for (int o = 1; o < 32; o <<= 1) {
    const int z = __shfl_up_sync(0xffffffffu, y, o);
    if (lane >= o) y += z;
  }
  const unsigned hit2 = __ballot_sync(0xffffffffu, y >= mr);
  if (!hit2) return -1;
  const int L2 = __ffs(hit2) - 1;
  const int k = mr - __shfl_sync(0xffffffffu, y - wc, L2);
  const unsigned ww = __shfl_sync(0xffffffffu, w, L2);
  const bool set = (ww >> lane) & 1u;
  const int below = __popc(ww & ((1u << lane) - 1u));
  const unsigned hit3 = __ballot_sync(0xffffffffu, set && below == k - 1);
  if (!hit3) return -1;
  return (gg * 32 + L2) * 32 + (__ffs(hit3) - 1);
}

// First member position >= from (INT_MAX if none) / last member position
// <= from (-1 if none); one warp.
__device__ int warp_next_member(const unsigned* wm, int from, int ng) {
  const int lane = threadIdx.x & 31;
  if (from >= ng) return INT_MAX;
  const int wlast = (ng - 1) >> 5;
  for (int w0 = from >> 5; w0 <= wlast; w0 += 32) {
    const int wi = w0 + lane;
    unsigned w = wi <= wlast ? wm[wi] : 0u;
    if (wi == (from >> 5)) w &= 0xffffffffu << (from & 31);
    const unsigned hit = __ballot_sync(0xffffffffu, w != 0u);
    if (hit) {
      const int L = __ffs(hit) - 1;
      const unsigned ww = __shfl_sync(0xffffffffu, w, L);
      const int pos = (w0 + L) * 32 + __ffs(ww) - 1;
      return pos < ng ? pos : INT_MAX;
    }
  }
  return INT_MAX;
}

__device__ int warp_prev_member(const unsigned* wm, int from) {
  const int lane = threadIdx.x & 31;
  if (from < 0) return -1;
  for (int w0 = from >> 5; w0 >= 0; w0 -= 32) {
    const int wi = w0 - lane;
    unsigned w = wi >= 0 ? wm[wi] : 0u;
    if (wi == (from >> 5)) {
      const int b = from & 31;
      w &= b == 31 ? 0xffffffffu : ((1u << (b + 1)) - 1u);
    }
    const unsigned hit = __ballot_sync(0xffffffffu, w != 0u);
    if (hit) {
      const int L = __ffs(hit) - 1;
      const unsigned ww = __shfl_sync(0xffffffffu, w, L);
      return (w0 - L) * 32 + 31 - __clz(ww);
    }
  }
  return -1;
}

// Whether hs slot j was deleted by a trial before trial i (before == true)
// or at any trial of this call (before == false).
__device__ __forceinline__ bool deleted_by(const GcmcSm& S, int j, int i, bool before) {
  for (int q = 0; q < S.ndel; ++q)
    if (S.del_slot[q] == j && (!before || S.del_trial[q] < i)) return true;
  return false;
}

// The rows that insertion k appends its atom to (ngroup_sort_atom,
// Neighbor.F90:303-317): hs%ref members within rc + skin of its point, at
// most one entry per row, among the 27 stencil cells: this call's earlier
// insertions, then the cell atoms.  Rows of atoms deleted in this call end
// empty and are skipped.  fn(j) is called by the lane holding target j.
template <class Fn>
__device__ void gcmc_append_targets(const Dev& d, const KParams& p, const RepConst& R,
                                    const GcmcSm& S, const GcmcTrialPre* pre, int k, Fn fn) {
  const int lane = threadIdx.x & 31;
  const GcmcTrialPre& tr = pre[S.ins_trial[k]];
  const double4 Rt = tr.r;
  const unsigned dup = tr.dup;
  const int mycell = lane < 27 ? tr.cells[lane] : -1;
  // at least 3 cells along every axis: the stencil index from the offsets
  const bool small = R.ncells[0] < 3 || R.ncells[1] < 3 || R.ncells[2] < 3;
  int t1 = 0, t2 = 0, t3 = 0;
  if (!small) cell_coords(R, tr.cell, t1, t2, t3);
  for (int k0 = 0; k0 < k; k0 += 32) {
    const int k2 = k0 + lane;
    const bool valid = k2 < k && S.ins_del[k2] == INT_MAX;
    const int c2 = valid ? S.ins_cell[k2] : -2;
    bool in = false;
    if (!small) {
      if (valid) {
        int a1, a2, a3;
        cell_coords(R, c2, a1, a2, a3);
        in = stencil_index_of(R, t1, t2, t3, a1, a2, a3) >= 0;
      }
    } else {
      for (int q = 0; q < 27; ++q) {
        const int cq = __shfl_sync(0xffffffffu, mycell, q);
        in |= valid && cq == c2 && !((dup >> q) & 1u);
      }
    }
    if (in) {
      double vx, vy, vz;
      vdist_nint(R, pre[S.ins_trial[k2]].r, Rt, vx, vy, vz);
      if (!(dot3(vx, vy, vz) > p.rlist2)) fn(R.base + S.ins_slot[k2]);
    }
  }
  const int nc = tr.n_cand;
  for (int c = lane; c < nc; c += 32) {
    if (!(tr.cf[c] & 2)) continue;
    const int j = tr.cand[c];
    if (!deleted_by(S, j, 0, false)) fn(j);
  }
}

__global__ void __launch_bounds__(kGcmcFastThreads)
    gcmc_fast_kernel(Dev d, KParams p, int wmax, int gmax, int words_smem) {
  DML_GRID_WAIT();
  const int rep = blockIdx.x;
  const GcmcRepPre* const gr = d.grp + rep;
  if (!gr->fast) return;
  if (threadIdx.x == 0) d.pr_cnt[rep * kCntStride + kCntGcmcPar] += 1;
  extern __shared__ double4 s_dyn[];
  GcmcSm& S = *reinterpret_cast<GcmcSm*>(s_dyn);
  int* const grp = reinterpret_cast<int*>(reinterpret_cast<char*>(s_dyn) + sizeof(GcmcSm));
  const RepConst& R = d.rc[rep];
  Scalars* const sc_g = d.sc + rep;
  const int B = R.base, tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, wid = tid >> 5;
  const int nw = nt >> 5;
  const GcmcTrialPre* const pre = d.gpre + (size_t)rep * kGcmcMaxTrials;
  const unsigned* const pmg = d.gpm + (size_t)rep * kGcmcMaxTrials * kGcmcMaskW;
  const int ng0 = gr->ng;
  const int nwords = min((ng0 + p.nadj + 63) >> 5, R.cap >> 5);
  const int ngrp = (nwords + 31) >> 5;
  unsigned *wm = d.gw_mem + B / 32, *wsl = d.gw_slab + B / 32;
  if (words_smem) {
    unsigned* sw = reinterpret_cast<unsigned*>(grp + gmax);
    for (int w = tid; w < nwords; w += nt) {
      sw[w] = wm[w];
      sw[wmax + w] = wsl[w];
    }
    wm = sw;
    wsl = sw + wmax;
  }
  if (tid == 0) {
    S.ss = *sc_g;
    S.nholes = gr->n_holes;
    S.nbholes = gr->n_bholes;
    S.napp = 0;
    S.app_over = 0;
  }
  for (int i = tid; i < p.nadj; i += nt) {
    const GcmcTrialPre& tr = pre[i];
    S.crt[i] = tr.coin < 0.5;
    S.rin[i] = in_slab(tr.r.z, sc_g->z0, sc_g->zmax);
    S.uacc[i] = tr.uacc;
    S.kpick[i] = tr.kpick;
    S.nblk[i] = tr.coin < 0.5 ? tr.n_blk : 0;
  }
  for (int e = tid; e < p.nadj * kGcmcBlk; e += nt) {
    const int i = e / kGcmcBlk, q = e - i * kGcmcBlk;
    S.blk[i][q] = pre[i].blk[q];
  }
  for (int e = tid; e < p.nadj * kGcmcMaskW; e += nt) S.pm[e / kGcmcMaskW][e % kGcmcMaskW] = pmg[e];
  for (int e = tid; e < kGcmcMaxTrials; e += nt) {
    S.holes[e] = gr->holes[e];
    S.bholes[e] = gr->bholes[e];
  }
  if (tid < kGcmcMaskW) S.acc[tid] = 0u;
  __syncthreads();
  // in-slab members per 1024 positions
  for (int g = wid; g < ngrp; g += nw) {
    const int wi = g * 32 + lane;
    int c = wi < nwords ? __popc(wsl[wi]) : 0;
    for (int off = 16; off > 0; off >>= 1) c += __shfl_down_sync(0xffffffffu, c, off);
    if (lane == 0) grp[g] = c;
  }
  __syncthreads();

  // Acceptance quotients for every control-volume count the call can reach
  // (n0 - nadj .. n0 + nadj), the same expressions as the sequential search.
  const int n0 = gr->n_in, qb = n0 - p.nadj;
  {
    const double v = R.box[0] * R.box[1] * (S.ss.zmax - S.ss.z0);
    for (int t = tid; t <= 2 * p.nadj; t += nt) {
      const int n = qb + t;
      S.qc[t] = p.act * v / (double)(n + 1);  // creation (dana.F90:630)
      S.qd[t] = (double)n / (v * p.act);      // destruction (dana.F90:683)
    }
  }
  __syncthreads();

  // The trials in order (dana.F90:620-710), one warp, shared state only.
  // hs%b slots, which no decision reads, are assigned afterwards.
  if (wid == 0) {
    // in-slab members up to and including 1024-position group g, for g =
    // lane (P0) and lane + 32 (P1): the first step of the deletion pick
    const bool reg_sel = ngrp <= 64;
    int P0 = 0, P1 = 0;
    if (reg_sel) {
      P0 = lane < ngrp ? grp[lane] : 0;
      P1 = lane + 32 < ngrp ? grp[lane + 32] : 0;
      for (int o = 1; o < 32; o <<= 1) {
        const int y0 = __shfl_up_sync(0xffffffffu, P0, o), y1 = __shfl_up_sync(0xffffffffu, P1, o);
        if (lane >= o) {
          P0 += y0;
          P1 += y1;
        }
      }
      P1 += __shfl_sync(0xffffffffu, P0, 31);
    }
    int n = n0, first = gr->first, last = gr->last, ng = ng0;
    int ns = S.ss.n_slots, n_atoms = S.ss.n_atoms, nlimbo = S.ss.nlimbo;
    int free_lo = S.ss.free_lo;
    int n_alist = S.ss.n_alist, n_rank = S.ss.n_rank;
    long long next_id = S.ss.next_id;
    int hi = 0, nins = 0, ndel = 0;
    int err = 0, err_info = 0;
    for (int i = 0; i < p.nadj; ++i) {
      __syncwarp();
      const int t = i + 1;
      if (first == INT_MAX) {
        err = DML_E_NO_PARTICLES;
        err_info = t;
        break;
      }
      const double uacc = S.uacc[i];
      if (S.crt[i]) {
        // creation attempt (dana.F90:627-677)
        if (f64_lt(S.qc[n - qb], uacc)) continue;
        // a blocker still in the group (its membership bit), or an earlier
        // insertion of this call still in it
        bool ov = false;
        if (lane < S.nblk[i]) {
          const int bp = S.blk[i][lane];
          ov = (wm[bp >> 5] >> (bp & 31)) & 1u;
        }
        if (lane < kGcmcMaskW && (S.pm[i][lane] & S.acc[lane]) != 0u) ov = true;
        if (__any_sync(0xffffffffu, ov)) continue;
        // first free hs slot (limbo slots are not free)
        int lslot;
        if (ns >= n_atoms + 1 + nlimbo) {
          if (hi >= S.nholes) {
            err = DML_E_INDEX;
            err_info = t;
            break;
          }
          lslot = S.holes[hi++];
        } else {
          lslot = ns;
        }
        if (lslot >= R.cap || n_rank >= R.cap || n_alist >= R.cap || ng >= R.cap) {
          err = DML_E_CAPACITY;
          err_info = t;
          break;
        }
        if (lane == 0) {
          S.ins_trial[nins] = i;
          S.ins_slot[nins] = lslot;
          S.ins_fpos[nins] = first;
          S.ins_lpos[nins] = last;
          S.ins_gpos[nins] = ng;
          S.ins_rank[nins] = n_rank;
          S.ins_alist[nins] = n_alist;
          S.ins_id[nins] = next_id;
          S.ins_del[nins] = INT_MAX;
          S.pos2ins[ng - ng0] = nins;
          wm[ng >> 5] |= 1u << (ng & 31);
          if (S.rin[i]) {
            wsl[ng >> 5] |= 1u << (ng & 31);
            grp[ng >> 10] += 1;
          }
          S.acc[i >> 5] |= 1u << (i & 31);
        }
        if (S.rin[i]) {
          const int g = ng >> 10;
          P0 += lane >= g;
          P1 += lane + 32 >= g;
        }
        n += 1;
        last = ng;
        ng += 1;
        n_alist += 1;
        n_rank += 1;
        if (lslot == ns) ns += 1;
        free_lo = lslot + 1;
        n_atoms += 1;
        next_id += 1;
        nins += 1;
      } else {
        // destruction attempt (dana.F90:680-707)
        if (f64_lt(S.qd[n - qb], uacc)) continue;
        const int m = gcmc_pick_index(S.kpick[i], n);
        // m <= 0: the walk never reaches m == 0 and ends on the last member
        const int psel = m <= 0 ? last : (reg_sel ? warp_select_reg(wsl, P0, P1, ng, m)
                                                  : warp_select(wsl, grp, ng, m));
        if (psel < 0) {
          err = DML_E_CHOSEN_MISSING;
          err_info = t;
          break;
        }
        const int kins = psel >= ng0 ? S.pos2ins[psel - ng0] : -1;
        // lane 0's reading, taken before it clears the bit, for every lane
        const bool was_in =
            __shfl_sync(0xffffffffu, (int)((wsl[psel >> 5] >> (psel & 31)) & 1u), 0) != 0;
        if (lane == 0) {
          S.del_trial[ndel] = i;
          S.del_pos[ndel] = psel;
          S.del_kins[ndel] = kins;
          if (kins >= 0) {
            S.ins_del[kins] = i;
            const int ti = S.ins_trial[kins];
            S.acc[ti >> 5] &= ~(1u << (ti & 31));
          }
          wm[psel >> 5] &= ~(1u << (psel & 31));
          if (was_in) {
            wsl[psel >> 5] &= ~(1u << (psel & 31));
            grp[psel >> 10] -= 1;
          }
        }
        if (was_in) {
          const int g = psel >> 10;
          P0 -= lane >= g;
          P1 -= lane + 32 >= g;
        }
        ndel += 1;
        nlimbo += 1;
        n_atoms -= 1;
        n -= 1;
        __syncwarp();
        // new first / last member when one of them left the group
        if (psel == first) first = warp_next_member(wm, psel + 1, ng);
        if (psel == last) last = warp_prev_member(wm, psel - 1);
      }
    }
    __syncwarp();
    if (lane == 0) {
      if (err) raise_error(d.g, err, err_info);
      S.nins = nins;
      S.ndel = ndel;
      S.ss.n_slots = ns;
      S.ss.n_atoms = n_atoms;
      S.ss.nlimbo = nlimbo;
      S.ss.free_lo = free_lo;
      S.ss.n_alist = n_alist;
      S.ss.n_rank = n_rank;
      S.ss.n_gorder = ng;
      S.ss.next_id = next_id;
      S.ss.n_ref += nins;
      S.ss.n_gcmc += nins - ndel;
      S.ss.gcmc_ins += (unsigned long long)nins;
      S.ss.gcmc_del += (unsigned long long)ndel;
      S.ss.halo = 0;
    }
  }
  __syncthreads();
  const int nins = S.nins, ndel = S.ndel;
  for (int k = tid; k < nins; k += nt) S.ins_cell[k] = pre[S.ins_trial[k]].cell;
  // the deleted atoms' hs and hs%b slots
  for (int q = tid; q < ndel; q += nt) {
    const int kins = S.del_kins[q];
    if (kins >= 0) {
      S.del_slot[q] = B + S.ins_slot[kins];
    } else {
      const int h = d.gorder[B + S.del_pos[q]];
      S.del_slot[q] = h;
      S.del_bslot[q] = d.bslot[h] - B;
    }
  }
  __syncthreads();
  // Three independent parts at once: warp 0 assigns the hs%b slots, warp 1
  // resolves the templates and Maxwell velocities, the other warps write the
  // inserted atoms' own lists.
  if (wid == 0) {
    // hs%b slots (cgroup_attach_atom, Cells.F90:105-144, and igroup's first
    // free slot) in trial order: an insertion takes the lower of the next
    // original hole and the lowest slot freed by an earlier deletion of this
    // call (a min-heap), or appends when there is no hole.
    if (lane == 0) {
      int nb = S.ss.n_b, b_nat = S.ss.b_nat, bfree_lo = S.ss.bfree_lo, bhi = 0, nh = 0;
      int a = 0, b = 0;
      bool bad = false;
      while (a < nins || b < ndel) {
        if (b >= ndel || (a < nins && S.ins_trial[a] < S.del_trial[b])) {
          int lbs = -1;
          if (nb >= b_nat + 1) {
            const int co = bhi < S.nbholes ? S.bholes[bhi] : INT_MAX;
            const int fm = nh > 0 ? S.freed[0] : INT_MAX;
            if (co == INT_MAX && fm == INT_MAX) {
              if (!bad) raise_error(d.g, DML_E_INDEX, S.ins_trial[a] + 1);
              bad = true;
            } else if (co < fm) {
              lbs = co;
              ++bhi;
            } else {
              lbs = fm;
              S.del_reused[S.freed_del[0]] = 1;
              // pop the heap root
              --nh;
              int vx = S.freed[nh], vd = S.freed_del[nh], x = 0;
              for (;;) {
                int c = 2 * x + 1;
                if (c >= nh) break;
                if (c + 1 < nh && S.freed[c + 1] < S.freed[c]) ++c;
                if (S.freed[c] >= vx) break;
                S.freed[x] = S.freed[c];
                S.freed_del[x] = S.freed_del[c];
                x = c;
              }
              S.freed[x] = vx;
              S.freed_del[x] = vd;
            }
          } else {
            lbs = nb;
          }
          if (lbs >= R.cap) {
            if (!bad) raise_error(d.g, DML_E_CAPACITY, S.ins_trial[a] + 1);
            bad = true;
            lbs = -1;
          }
          S.ins_bslot[a] = lbs;
          if (lbs >= 0) {
            if (lbs == nb) nb += 1;
            b_nat += 1;
            bfree_lo = lbs + 1;
          }
          ++a;
        } else {
          const int kins = S.del_kins[b];
          const int bsl = kins >= 0 ? S.ins_bslot[kins] : S.del_bslot[b];
          S.del_bslot[b] = bsl;
          S.del_reused[b] = 0;
          if (bsl >= 0) {
            // push on the heap
            int x = nh++;
            while (x > 0 && S.freed[(x - 1) / 2] > bsl) {
              S.freed[x] = S.freed[(x - 1) / 2];
              S.freed_del[x] = S.freed_del[(x - 1) / 2];
              x = (x - 1) / 2;
            }
            S.freed[x] = bsl;
            S.freed_del[x] = b;
            if (bsl < bfree_lo) bfree_lo = bsl;
            b_nat -= 1;
          }
          ++b;
        }
      }
      S.ss.n_b = nb;
      S.ss.b_nat = b_nat;
      S.ss.bfree_lo = bfree_lo;
    }
  } else if (wid == 1) {
    // Templates (the first member) and Maxwell targets (the last member) of
    // the insertions, as hs slots; pre-call values of the pre-call atoms.
    for (int k = lane; k < nins; k += 32) {
      const int fp = S.ins_fpos[k], lp = S.ins_lpos[k];
      int hr, hri, hl, hli;
      if (fp >= ng0) {
        hri = S.pos2ins[fp - ng0];
        hr = B + S.ins_slot[hri];
      } else {
        hri = -1;
        hr = d.gorder[B + fp];
      }
      if (lp >= ng0) {
        hli = S.pos2ins[lp - ng0];
        hl = B + S.ins_slot[hli];
      } else {
        hli = -1;
        hl = d.gorder[B + lp];
      }
      S.href[k] = hr;
      S.href_ins[k] = hri;
      S.hlast[k] = hl;
      S.hlast_ins[k] = hli;
      if (hri < 0) {
        // the velocity (chosen form: the first half of the slot, two doubles)
        const double4 v0 = d.vel[hr];
        S.tvel[k] = Vel3{v0.x, v0.y, p.mixed ? 0.0 : v0.z};
        S.htyp[k] = d.typ[hr];
      }
      const GcmcTrialPre& tr = pre[S.ins_trial[k]];
      S.nv[k] = make_float4((float)tr.nv[0], (float)tr.nv[1], (float)tr.nv[2], 0.0f);
    }
    __syncwarp();
    // atom_asign copies the template's velocity, then the Maxwell velocity
    // goes to the last member (dana.F90:659-668): resolved in trial order.
    if (lane == 0) {
      int nmw = 0;
      for (int k = 0; k < nins; ++k) {
        const int hri = S.href_ins[k];
        Vel3 tv;
        int typ;
        if (hri >= 0) {
          S.root[k] = S.root[hri];
          typ = S.ityp[hri];
          tv = S.fvel[hri];
        } else {
          S.root[k] = S.href[k];
          typ = S.htyp[k];
          tv = S.tvel[k];
          for (int q = nmw - 1; q >= 0; --q)
            if (S.mw_slot[q] == S.href[k]) {
              tv = S.mw_vel[q];
              break;
            }
        }
        S.ityp[k] = typ;
        S.tvel[k] = tv;
        S.fvel[k] = tv;
        const double beta = p.beta_t[typ - 1];
        const float4 nv = S.nv[k];
        Vel3 mv = Vel3{beta * (double)nv.x, beta * (double)nv.y, beta * (double)nv.z};
        if (p.mixed) {  // the velocity half of the slot holds FP32 values (chosen form)
          const double4 pk = pack_f3((float)mv.x, (float)mv.y, (float)mv.z);
          mv = Vel3{pk.x, pk.y, 0.0};
        }
        const int hli = S.hlast_ins[k];
        if (hli >= 0) {
          S.fvel[hli] = mv;
        } else {
          int q = 0;
          while (q < nmw && S.mw_slot[q] != S.hlast[k]) ++q;
          if (q == nmw) {
            S.mw_slot[q] = S.hlast[k];
            nmw += 1;
          }
          S.mw_vel[q] = mv;
        }
      }
      S.n_mw = nmw;
    }
  } else {
    // Own lists (ngroup_cells_atom, Neighbor.F90:550-603): per stencil cell,
    // this call's earlier insertions in that cell (chain heads, most recent
    // first), then the sorted cell; atoms deleted before the trial left.
    // fewer than 3 cells along an axis: stencil cells repeat (general walk)
    const bool R_small = R.ncells[0] < 3 || R.ncells[1] < 3 || R.ncells[2] < 3;
    for (int k = wid - 2; k < nins; k += nw - 2) {
      if (S.ins_del[k] != INT_MAX) continue;  // deleted later: its row ends empty
      const int i = S.ins_trial[k];
      const GcmcTrialPre& tr = pre[i];
      const double4 Rt = tr.r;
      const int slot = B + S.ins_slot[k];
      int* row = d.list + (size_t)slot * p.mnb;
      const int mycell = lane < 27 ? tr.cells[lane] : -1;
      // the trial's candidates, two per lane (c = lane, lane + 32), in stencil
      // order: stencil index, and whether it joins the own list
      const int nc = tr.n_cand;
      int cj[2], cqq[2];
      bool cown[2];
  #pragma unroll
      for (int h2 = 0; h2 < 2; ++h2) {
        const int c = lane + 32 * h2;
        cj[h2] = c < nc ? tr.cand[c] : -1;
        cqq[h2] = c < nc ? (int)tr.cq[c] : -1;
        cown[h2] = c < nc && (tr.cf[c] & 1) && !deleted_by(S, cj[h2], i, true);
      }
      int cnt = 0;
      if (!R_small && k <= 64) {
        // each earlier insertion's stencil index (k2 = k - 1 - lane - 32 h2,
        // most recent first), -1 when outside the stencil, deleted before
        // the trial or beyond rc + skin; then the stencil walk by ballots
        int eq[2], ej[2];
        int t1, t2, t3;
        cell_coords(R, tr.cell, t1, t2, t3);
  #pragma unroll
        for (int h2 = 0; h2 < 2; ++h2) {
          const int k2 = k - 1 - lane - 32 * h2;
          eq[h2] = -1;
          ej[h2] = -1;
          if (k2 >= 0 && S.ins_del[k2] > i) {
            int a1, a2, a3;
            cell_coords(R, S.ins_cell[k2], a1, a2, a3);
            const int q = stencil_index_of(R, t1, t2, t3, a1, a2, a3);
            if (q >= 0) {
              double vx, vy, vz;
              vdist_nint(R, pre[S.ins_trial[k2]].r, Rt, vx, vy, vz);
              if (dot3(vx, vy, vz) < p.rlist2) {
                eq[h2] = q;
                ej[h2] = B + S.ins_slot[k2];
              }
            }
          }
        }
        for (int q = 0; q < 27; ++q) {
  #pragma unroll
          for (int h2 = 0; h2 < 2; ++h2) {
            const bool inc = eq[h2] == q;
            const unsigned bal = __ballot_sync(0xffffffffu, inc);
            const int pos = cnt + __popc(bal & ((1u << lane) - 1u));
            if (inc && pos < p.mnb) row[pos] = ej[h2];
            cnt += __popc(bal);
          }
  #pragma unroll
          for (int h2 = 0; h2 < 2; ++h2) {
            const bool inc = cown[h2] && cqq[h2] == q;
            const unsigned bal = __ballot_sync(0xffffffffu, inc);
            const int pos = cnt + __popc(bal & ((1u << lane) - 1u));
            if (inc && pos < p.mnb) row[pos] = cj[h2];
            cnt += __popc(bal);
          }
        }
      } else
      for (int q = 0; q < 27; ++q) {
        const int cq = __shfl_sync(0xffffffffu, mycell, q);
        for (int kb = k - 1; kb >= 0; kb -= 32) {
          const int k2 = kb - lane;
          bool inc = false;
          int j = -1;
          if (k2 >= 0 && S.ins_cell[k2] == cq && S.ins_del[k2] > i) {
            j = B + S.ins_slot[k2];
            double vx, vy, vz;
            vdist_nint(R, pre[S.ins_trial[k2]].r, Rt, vx, vy, vz);
            inc = dot3(vx, vy, vz) < p.rlist2;
          }
          const unsigned bal = __ballot_sync(0xffffffffu, inc);
          const int pos = cnt + __popc(bal & ((1u << lane) - 1u));
          if (inc && pos < p.mnb) row[pos] = j;
          cnt += __popc(bal);
        }
  #pragma unroll
        for (int h2 = 0; h2 < 2; ++h2) {
          const bool inc = cown[h2] && cqq[h2] == q;
          const unsigned bal = __ballot_sync(0xffffffffu, inc);
          const int pos = cnt + __popc(bal & ((1u << lane) - 1u));
          if (inc && pos < p.mnb) row[pos] = cj[h2];
          cnt += __popc(bal);
        }
      }
      if (lane == 0) {
        if (cnt > p.mnb) raise_error(d.g, DML_E_NEIGH_OVERFLOW, slot);
        d.nn[slot] = cnt > p.mnb ? p.mnb : cnt;
        list_new_row(d, slot);  // an inserted atom's row, written between full force scans
      }
    }
  }
  __syncthreads();
  // the inserted atoms (atom_asign and the attach loop, dana.F90:659-675)
  for (int k = tid; k < nins; k += nt) {
    const int slot = B + S.ins_slot[k], bs = B + S.ins_bslot[k];
    const int root = S.root[k], typ = S.ityp[k];
    const double4 tf = d.force[root], ta = d.acel[root];
    const double te = d.epot[root];
    const double4 Rt = pre[S.ins_trial[k]].r;
    if (p.mixed) {  // velocity resolved above, acceleration of the template
      const double4 tva = d.vel[root];
      d.vel[slot] = make_double4(S.fvel[k].x, S.fvel[k].y, tva.z, tva.w);
    } else {
      d.vel[slot] = make_double4(S.fvel[k].x, S.fvel[k].y, S.fvel[k].z, 0.0);
    }
    d.force[slot] = tf;
    if (p.mixed) atomicOr(&d.fnz[slot >> 5], 1u << (slot & 31));
    d.acel[slot] = ta;
    d.epot[slot] = te;
    d.typ[slot] = (int8_t)typ;
    d.pos[slot] = Rt;
    d.pos_old[slot] = Rt;
    d.posf_old[slot] = make_float4((float)Rt.x, (float)Rt.y, (float)Rt.z, 0.0f);
    d.old_cg[slot] = make_double4(1e8, 1e8, 1e8, 0.0);
    d.posf[slot] = to_f4(Rt, typ);
    d.skip[slot] = 0;
    d.id[slot] = S.ins_id[k];
    d.ev_count[slot] = 0;
    d.alist[B + S.ins_alist[k]] = slot;
    d.apos[slot] = B + S.ins_alist[k];
    d.ref[B + S.ins_rank[k]] = slot;
    d.rank[slot] = B + S.ins_rank[k];
    // an atom deleted later in this call leaves its hs%b slot to the
    // insertion that reuses it, or to the deletion that empties it
    if (S.ins_del[k] == INT_MAX && S.ins_bslot[k] >= 0) d.b2hs[bs] = slot;
    d.bslot[slot] = S.ins_bslot[k] >= 0 ? bs : -1;
    d.state[slot] = ST_LIVE;
    d.gorder[B + S.ins_gpos[k]] = slot;
    d.gpos[slot] = B + S.ins_gpos[k];
    d.in_gcmc[slot] = 1;
  }
  for (int q = tid; q < S.n_mw; q += nt) {
    if (p.mixed)  // the velocity half only
      *reinterpret_cast<double2*>(d.vel + S.mw_slot[q]) = make_double2(S.mw_vel[q].x, S.mw_vel[q].y);
    else
      d.vel[S.mw_slot[q]] = make_double4(S.mw_vel[q].x, S.mw_vel[q].y, S.mw_vel[q].z, 0.0);
  }
  __syncthreads();
  // the deleted atoms (atom_destroy: gcmc, hs (nn, hs%ref, hs%b), sys,
  // Groups.F90:433-467); a freed hs%b slot that a later insertion took keeps it
  for (int q = tid; q < ndel; q += nt) {
    const int h = S.del_slot[q];
    const int rk = d.rank[h], ap = d.apos[h];
    const float4 pf = d.posf[h];
    d.in_gcmc[h] = 0;
    d.gorder[B + S.del_pos[q]] = -1;
    d.nn[h] = 0;
    if (rk >= 0) {
      d.ref[rk] = -1;
      d.rank[h] = -1;
      atomicSub(&S.ss.n_ref, 1);
    }
    if (!S.del_reused[q] && S.del_bslot[q] >= 0) d.b2hs[B + S.del_bslot[q]] = -1;
    d.bslot[h] = -1;
    d.state[h] = ST_LIMBO;
    d.posf[h] = make_float4(pf.x, pf.y, pf.z, __int_as_float(0));
    d.alist[ap] = -1;
  }
  __syncthreads();
  // Appends (ngroup_sort_atom): row j receives the atoms of the insertions
  // that reach it, in trial order, after what it holds.
  for (int k = wid; k < nins; k += nw)
    gcmc_append_targets(d, p, R, S, pre, k, [&](int j) {
      const int e = atomicAdd(&S.napp, 1);
      if (e < kGcmcAppCap) {
        S.app_j[e] = j;
        S.app_k[e] = k;
      } else {
        S.app_over = 1;
      }
    });
  __syncthreads();
  if (!S.app_over) {
    const int na = S.napp;
    for (int e = tid; e < na; e += nt) S.app_base[e] = d.nn[S.app_j[e]];
    __syncthreads();
    for (int e = tid; e < na; e += nt) {
      const int j = S.app_j[e], k = S.app_k[e];
      int before = 0, cnt = 0;
      for (int f = 0; f < na; ++f)
        if (S.app_j[f] == j) {
          cnt += 1;
          before += S.app_k[f] < k;
        }
      const int m = S.app_base[e] + before;
      if (m < p.mnb) d.list[(size_t)j * p.mnb + m] = B + S.ins_slot[k];
      else raise_error(d.g, DML_E_NEIGH_OVERFLOW, j);
      if (before == cnt - 1) {
        d.nn[j] = min(S.app_base[e] + cnt, p.mnb);
        flag_row(d, j);
      }
    }
  } else if (wid == 0) {
    // more appends than the shared table holds: one insertion at a time
    for (int k = 0; k < nins; ++k) {
      gcmc_append_targets(d, p, R, S, pre, k, [&](int j) {
        const int m = d.nn[j];
        if (m >= p.mnb) {
          raise_error(d.g, DML_E_NEIGH_OVERFLOW, j);
          return;
        }
        d.list[(size_t)j * p.mnb + m] = B + S.ins_slot[k];
        d.nn[j] = m + 1;
        flag_row(d, j);
      });
      __syncwarp();
    }
  }
  __syncthreads();
  if (tid == 0) *sc_g = S.ss;
}

// dml_set_atoms_batch on the device: the replica of every position, then
// every loaded atom's slot (hs slot = hs%b slot = sys%alist position) from
// the compact input.  Positions left unused keep the -1 / zero fill.
__global__ void load_rep_kernel(Dev d) {
  DML_GRID_WAIT();
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < d.cap; q += gridDim.x * blockDim.x) {
    int lo = 0, hi = d.nrep - 1;  // largest replica whose base is <= q
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (d.rc[mid].base <= q) lo = mid; else hi = mid - 1;
    }
    d.rep_of[q] = lo;
  }
}

__global__ void load_atoms_kernel(Dev d, KParams p, LoadIn in) {
  DML_GRID_WAIT();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < in.n_tot; i += gridDim.x * blockDim.x) {
    int lo = 0, hi = d.nrep - 1;  // replica of compact atom i
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (in.off[mid] <= i) lo = mid; else hi = mid - 1;
    }
    const int li = i - in.off[lo], B = d.rc[lo].base, h = B + li;
    auto v3 = [&](const double* a, double def) {
      return a ? make_double4(a[3 * i], a[3 * i + 1], a[3 * i + 2], 0.0)
               : make_double4(def, def, def, 0.0);
    };
    const int z = in.z[i];
    const double4 P = v3(in.pos, 0.0);
    const double4 O = in.pos_old ? v3(in.pos_old, 0.0) : P;
    d.pos[h] = P;
    d.pos_old[h] = O;
    d.posf[h] = to_f4(P, z);
    d.posf_old[h] = to_f4(O, 0);
    const double4 V = v3(in.vel, 0.0), A = v3(in.acel, 0.0);
    if (p.mixed) {  // FP32 velocity and acceleration in one slot (chosen form)
      float4* q = reinterpret_cast<float4*>(d.vel + h);
      q[0] = make_float4((float)V.x, (float)V.y, (float)V.z, 0.0f);
      q[1] = make_float4((float)A.x, (float)A.y, (float)A.z, 0.0f);
    } else {
      d.vel[h] = V;
      d.acel[h] = A;
    }
    d.force[h] = v3(in.force, 0.0);
    d.old_cg[h] = v3(in.old_cg, 1e8);
    d.epot[h] = in.epot ? in.epot[i] : 0.0;
    d.typ[h] = (int8_t)z;
    d.skip[h] = in.skip ? (int8_t)(in.skip[i] != 0) : (int8_t)0;
    d.state[h] = ST_LIVE;
    d.id[h] = in.id ? in.id[i] : (long long)li;
    d.alist[h] = h;
    d.apos[h] = h;
    d.bslot[h] = h;
    d.b2hs[h] = h;
    const int rk = in.rk[i], gk = in.gk[i];
    if (rk >= 0) {
      if (z == DML_Z_F) note_f(d, h);  // committed at the first capture commit
      d.rank[h] = B + rk;
      d.ref[B + rk] = h;
    }
    if (gk >= 0) {
      d.gpos[h] = B + gk;
      d.gorder[B + gk] = h;
      d.in_gcmc[h] = 1;
    }
  }
}

inline int nblk(int n, int b = kBlock) { return n > 0 ? (n + b - 1) / b : 1; }
// blocks of the per-position kernels over n positions (a multiple of kSpan)
inline int nspan(int n) { return n > 0 ? (n + kSpan - 1) / kSpan : 1; }
inline int nblk_warps(int n) { return n > 0 ? (n + (kBlock / 32) - 1) / (kBlock / 32) : 1; }
// Fixed grid of the warp-per-row kernels (grid-stride over the rows): a
// few resident blocks per SM instead of one block per 8 rows.
constexpr int kRowGrid = 152 * 16;
inline int nblk_rows(int rows) { int b = nblk_warps(rows); return b < kRowGrid ? b : kRowGrid; }

// Overwrites a buffer larger than L2 (benchmark L2 flush between steps).
__global__ void flush_kernel(uint4* buf, size_t n) {
  DML_GRID_WAIT();
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  size_t stride = (size_t)gridDim.x * blockDim.x;
  for (; i < n; i += stride) buf[i] = make_uint4((unsigned)i, 0u, 0u, 0u);
}

}  // namespace

int k_step_begin(const Dev& d, int near_stale, cudaStream_t s) {
  step_begin_kernel<<<1, 256, 0, s>>>(d, near_stale);
  return 1;
}

int k_ermak_a(const Dev& d, const KParams& p, int n_rank, cudaStream_t s) {
  if (p.mixed)
    ermak_a_kernel<true><<<nspan(n_rank), kBlock, 0, s>>>(d, p, n_rank);
  else
    ermak_a_kernel<false><<<nspan(n_rank), kBlock, 0, s>>>(d, p, n_rank);
  return 1;
}

int k_brownian(const Dev& d, const KParams& p, int n_rank, cudaStream_t s) {
  if (p.mixed)
    brownian_kernel<true><<<nspan(n_rank), kBlock, 0, s>>>(d, p, n_rank);
  else
    brownian_kernel<false><<<nspan(n_rank), kBlock, 0, s>>>(d, p, n_rank);
  return 1;
}

template <bool NEAR>
void launch_force_scan(const Dev& d, const KParams& p, int n_rank, cudaStream_t s) {
  const int L = p.scan_lanes;
  const int nb = nblk_rows((n_rank + 32 / L - 1) / (32 / L));
  if (L == 1)
    force_scan_span_kernel<NEAR><<<nspan(n_rank), kBlock, 0, s>>>(d, p);
  else if (L == 2)
    force_scan_kernel<NEAR, 2><<<nb, kBlock, 0, s>>>(d, p);
  else if (L == 4)
    force_scan_kernel<NEAR, 4><<<nb, kBlock, 0, s>>>(d, p);
  else if (L == 8)
    force_scan_kernel<NEAR, 8><<<nb, kBlock, 0, s>>>(d, p);
  else if (L == 32)
    force_scan_kernel<NEAR, 32><<<nb, kBlock, 0, s>>>(d, p);
  else
    force_scan_kernel<NEAR, 16><<<nb, kBlock, 0, s>>>(d, p);
}

int k_force_scan(const Dev& d, const KParams& p, int n_rank, bool near, cudaStream_t s) {
  if (near)
    launch_force_scan<true>(d, p, n_rank, s);
  else
    launch_force_scan<false>(d, p, n_rank, s);
  return 1;
}

int k_force_pairs(const Dev& d, const KParams& p, int n_rank, bool near, cudaStream_t s) {
  int n = 2;
  if (near && p.short_scan) {
    scan_mode_kernel<<<1, 256, 0, s>>>(d, p);
    force_scan_listed_kernel<true><<<152 * 8, kBlock, 0, s>>>(d, p);
    n += 2;
  }
  k_force_scan(d, p, n_rank, near, s);
  if (p.mixed)
    force_exact_mixed_kernel<<<152 * 4, kBlock, 0, s>>>(d, p);
  else
    force_exact_kernel<<<152 * 4, kBlock, 0, s>>>(d, p);
  return n;
}

int k_scan_invalidate(const Dev& d, cudaStream_t s) {
  scan_invalidate_kernel<<<1, 256, 0, s>>>(d);
  return 1;
}

int k_reset_candidates(const Dev& d, cudaStream_t s) {
  return cudaMemsetAsync(&d.g->n_cand, 0, sizeof(int), s) == cudaSuccess ? 0 : 1;
}

int k_force_sum(const Dev& d, const KParams& p, int n_slots, bool fuse_b, cudaStream_t s) {
  if (p.mixed) {
    // listed slots first: force_ref_kernel skips the members they summed
    // (and resets the list)
    if (fuse_b) {
      force_touched_kernel<true><<<152 * 2, kBlock, 0, s>>>(d, p);
      force_ref_kernel<true><<<nspan(n_slots), kBlock, 0, s>>>(d, p);
    } else {
      force_touched_kernel<false><<<152 * 2, kBlock, 0, s>>>(d, p);
      force_ref_kernel<false><<<nspan(n_slots), kBlock, 0, s>>>(d, p);
    }
    return 2;
  }
  if (fuse_b)
    force_sum_kernel<true><<<nspan(n_slots), kBlock, 0, s>>>(d, p, n_slots);
  else
    force_sum_kernel<false><<<nspan(n_slots), kBlock, 0, s>>>(d, p, n_slots);
  return 1;
}

int k_ermak_b(const Dev& d, const KParams& p, int n_rank, cudaStream_t s) {
  ermak_b_kernel<<<nspan(n_rank), kBlock, 0, s>>>(d, p, n_rank);
  return 1;
}

int k_pbc_dispmax(const Dev& d, const KParams& p, int n_slots, cudaStream_t s, bool second) {
  pbc_dispmax_kernel<<<nspan(n_slots), kBlock, 0, s>>>(d, p, n_slots, second ? 1 : 0);
  dispmax_exact_kernel<<<kExactGrid, kBlock, 0, s>>>(d, p, 0, 0);
  return 2;
}

int k_test_update(const Dev& d, const KParams& p, int n_slots, int n_b, int n_rank,
                  cudaStream_t s, bool second) {
  return k_pbc_dispmax(d, p, n_slots, s, second) + k_rebuild(d, p, n_slots, n_b, n_rank, s);
}

int k_pbc_dispmax_cond(const Dev& d, const KParams& p, int n_slots,
                       cudaGraphConditionalHandle h, cudaStream_t s, bool second) {
  pbc_dispmax_kernel<<<nspan(n_slots), kBlock, 0, s>>>(d, p, n_slots, second ? 1 : 0);
  dispmax_exact_kernel<<<kExactGrid, kBlock, 0, s>>>(d, p, 1, h);
  return 2;
}

int k_rebuild(const Dev& d, const KParams& p, int n_slots, int n_b, int n_rank, cudaStream_t s) {
  int nmax = n_slots > n_b ? n_slots : n_b;
  rebuild_prep_kernel<<<nspan(nmax), kBlock, 0, s>>>(d, p, n_slots, n_b, 0);
  int n = 1;
  if (d.any_cells) {
    // cell starts and in-cell order over the rebuilding replicas' chunks
    cell_chunk_sum_kernel<<<152 * 8, kBlock, 0, s>>>(d);
    cell_chunk_scan_kernel<<<d.nrep, 1024, 0, s>>>(d);
    cell_chunk_fill_kernel<<<152 * 8, kBlock, 0, s>>>(d);
    cell_scatter_kernel<<<nspan(n_b), kBlock, 0, s>>>(d, n_b, 0);
    cell_order_reb_kernel<<<152 * 8, kBlock, 0, s>>>(d);
    cell_order_big_kernel<<<152 * 4, kBlock, 0, s>>>(d, 0);
    n += 6;
    if (d.any_list_warp) {
      list_cells_kernel<<<nblk_rows(n_rank), kBlock, 0, s>>>(d, p, n_rank);
      n += 1;
    }
    if (d.any_list_thread) {
      list_cells_thread_kernel<<<nblk(n_rank) < kRowGrid ? nblk(n_rank) : kRowGrid, kBlock, 0,
                                 s>>>(d, p);
      n += 1;
    }
  }
  if (d.any_verlet) {
    list_verlet_kernel<<<nblk_rows(n_rank), kBlock, 0, s>>>(d, p, n_rank, n_b);
    n += 1;
  }
  rebuild_done_kernel<<<nblk(d.nrep), kBlock, 0, s>>>(d);
  return n + 1;
}

int k_overlap_prepare(const Dev& d, const KParams& p, int n_slots, cudaStream_t s) {
  overlap_init_kernel<<<nspan(n_slots), kBlock, 0, s>>>(d, p, n_slots);
  return 1;
}

int k_overlap_detect(const Dev& d, const KParams& p, int n_rank, int mode, cudaStream_t s) {
  const int L = p.near_lanes;
  const int nb = nblk_rows((n_rank + 32 / L - 1) / (32 / L));
  switch (L) {
    case 1: overlap_detect_kernel<1><<<nb, kBlock, 0, s>>>(d, p, mode); break;
    case 2: overlap_detect_kernel<2><<<nb, kBlock, 0, s>>>(d, p, mode); break;
    case 4: overlap_detect_kernel<4><<<nb, kBlock, 0, s>>>(d, p, mode); break;
    case 8: overlap_detect_kernel<8><<<nb, kBlock, 0, s>>>(d, p, mode); break;
    case 16: overlap_detect_kernel<16><<<nb, kBlock, 0, s>>>(d, p, mode); break;
    default: overlap_detect_kernel<32><<<nb, kBlock, 0, s>>>(d, p, mode); break;
  }
  return 1;
}

int k_rank_prefix(const Dev& d, cudaStream_t s) {
  rank_prefix_kernel<<<1, 1024, 0, s>>>(d);
  return 1;
}

int k_overlap(const Dev& d, const KParams& p, int n_rank, int n_slots, bool standalone,
              int detect, cudaStream_t s) {
  int n = 0;
  if (standalone) {
    delta_reset_kernel<<<1, 1, 0, s>>>(d.g);
    n += 1 + k_overlap_prepare(d, p, n_slots, s);
  }
  if (detect) n += k_overlap_detect(d, p, n_rank, detect == 1 ? 1 : 0, s);
  overlap_count_kernel<<<nspan(n_rank), kBlock, 0, s>>>(d, n_rank);
  overlap_big_prefix_kernel<<<1, 256, 0, s>>>(d);
  // replicas with many listed members: their bookkeeping on the whole grid
  overlap_assign_big_kernel<<<152 * 4, kBlock, 0, s>>>(d);
  overlap_scatter_big_kernel<<<152 * 4, kBlock, 0, s>>>(d);
  overlap_order_big_kernel<<<152 * 4, kBlock, 0, s>>>(d);
  const int all_passes = p.prob >= 1.0;
  // with prob >= 1 the passes of a replica with few components run inside
  // the per-replica kernel, the others in overlap_pass1_kernel
  overlap_comp_kernel<<<d.nrep, kCompThreads, 0, s>>>(d, p, all_passes);
  overlap_pass1_kernel<<<152 * 16, 128, 0, s>>>(d, p, all_passes);
  n += 7;
  if (all_passes) return n;
  overlap_passn_kernel<<<1, 1024, 0, s>>>(d, p);
  return n + 1;
}

int k_bloques(const Dev& d, const KParams& p, cudaStream_t s) {
  bloques_kernel<<<d.nrep, 32, 0, s>>>(d, p);
  return 1;
}

int k_chunk_cond(const Dev& d, cudaGraphConditionalHandle h, cudaStream_t s) {
  chunk_cond_kernel<<<1, 1, 0, s>>>(d.g, h);
  return 1;
}

int k_capture_commit(const Dev& d, const KParams& p, int n_rank, cudaStream_t s) {
  (void)p;
  (void)n_rank;
  commit_kernel<<<1, 1024, 0, s>>>(d);
  return 1;
}

int k_calc_rho(const Dev& d, const KParams& p, int n_slots, cudaStream_t s) {
  calc_rho_kernel<<<nspan(n_slots), kBlock, 0, s>>>(d, p, n_slots);
  return 1;
}

int k_piston(const Dev& d, const KParams& p, int n_slots, cudaStream_t s) {
  piston_kernel<<<nspan(n_slots), kBlock, 0, s>>>(d, p, n_slots);
  return 1;
}

// Whether gcmc_run's trials take the parallel path (gcmc_pre_kernel and
// gcmc_fast_kernel, for the replicas that qualify), with the dynamic shared
// memory of gcmc_fast_kernel and whether its bit words fit there.
struct GcmcLaunch {
  int par, wmax, gmax, words_smem;
  size_t fshm, pshm;
};
static GcmcLaunch gcmc_launch(const Dev& d, const KParams& p) {
  GcmcLaunch L;
  static_assert(sizeof(GcmcSm) <= 100 * 1024, "gcmc_fast_kernel shared state");
  L.wmax = d.max_rep_cap / 32;
  L.gmax = (L.wmax + 31) / 32 + 1;
  L.fshm = sizeof(GcmcSm) + sizeof(int) * (size_t)L.gmax;
  L.words_smem = L.fshm + 2 * sizeof(unsigned) * (size_t)L.wmax <= 200 * 1024;
  if (L.words_smem) L.fshm += 2 * sizeof(unsigned) * (size_t)L.wmax;
  L.pshm = sizeof(int) * (size_t)d.gcmc_rows;
  L.par = d.gpre != nullptr && d.grp != nullptr && p.nadj <= kGcmcMaxTrials &&
          L.fshm <= 220 * 1024 && d.gcmc_rows > 0;
  return L;
}

// gcmc_run's searches need the cells of the current positions: the
// preparation, then the listing of the atoms the trials can reach (and the
// parallel path's bit words).
int k_gcmc_cells(const Dev& d, const KParams& p, int cap, cudaStream_t s) {
  if (!d.any_cells) return 0;
  const GcmcLaunch L = gcmc_launch(d, p);
  gcmc_prep_kernel<<<d.nrep, 512, 0, s>>>(d, p, L.par);
  gcmc_bin_kernel<<<nspan(cap), kBlock, 0, s>>>(d, L.par);
  return 2;
}

int k_gcmc(const Dev& d, const KParams& p, int cap, cudaStream_t s) {
  return k_gcmc_cells(d, p, cap, s) + k_gcmc_trials(d, p, s);
}

// The trials: on the parallel path the per-replica searches, then the cell
// sort of the replicas that run sequentially (all of them otherwise), the
// parallel decisions and the sequential gcmc_kernel.
int k_gcmc_trials(const Dev& d, const KParams& p, cudaStream_t s) {
  int n = 0;
  const GcmcLaunch L = gcmc_launch(d, p);
  if (L.par) {
    cudaFuncSetAttribute(gcmc_pre_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.pshm);
    gcmc_pre_kernel<<<d.nrep, kGcmcPreThreads, L.pshm, s>>>(d, p);
    n += 1;
  }
  if (d.any_cells && L.par) {  // the replicas that run sequentially (usually none)
    gcmc_count_rep_kernel<<<d.nrep, kBlock, 0, s>>>(d);
    cell_scan_kernel<<<d.nrep, 1024, 0, s>>>(d, 1, 1);
    gcmc_scatter_rep_kernel<<<d.nrep, kBlock, 0, s>>>(d);
    gcmc_order_kernel<<<d.nrep, kBlock, 0, s>>>(d);
    cell_order_big_kernel<<<152 * 4, kBlock, 0, s>>>(d, 1);
    n += 5;
  } else if (d.any_cells) {  // all replicas
    const int cap = d.cap;
    gcmc_count_kernel<<<nspan(cap), kBlock, 0, s>>>(d, 0);
    cell_scan_kernel<<<d.nrep, 1024, 0, s>>>(d, 1, 0);
    gcmc_scatter_kernel<<<nspan(cap), kBlock, 0, s>>>(d, 0);
    cell_order_small_kernel<<<d.n_cch > 0 ? d.n_cch : 1, kBlock, 0, s>>>(d, 1, 0);
    cell_order_big_kernel<<<152 * 4, kBlock, 0, s>>>(d, 1);
    n += 5;
  }
  if (L.par) {
    cudaFuncSetAttribute(gcmc_fast_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.fshm);
    gcmc_fast_kernel<<<d.nrep, kGcmcFastThreads, L.fshm, s>>>(d, p, L.wmax, L.gmax, L.words_smem);
    n += 1;
  }
  size_t shm = sizeof(GcmcTrial) * (size_t)kGcmcTrialBatch +
               sizeof(int) * (size_t)(d.max_rep_cap / kGcmcThreads + 2);
  if (shm > 48 * 1024)
    cudaFuncSetAttribute(gcmc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
  gcmc_kernel<<<d.nrep, kGcmcThreads, shm, s>>>(d, p, L.par);
  return n + 1;
}

int k_flush(void* buf, size_t bytes, cudaStream_t s) {
  size_t n = bytes / sizeof(uint4);
  flush_kernel<<<152 * 8, 512, 0, s>>>((uint4*)buf, n);
  return 1;
}

}  // namespace dml

namespace dml {
__global__ void check_conversions_kernel(const double* x, float* f32, double* back,
                                         long long n) {
  DML_GRID_WAIT();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const float f = f64_to_f32_rn(x[i]);
    f32[i] = f;
    back[i] = f32_to_f64(f);
  }
}

__global__ void check_pick_kernel(const unsigned long long* k, const int* n, int* m,
                                  long long count) {
  DML_GRID_WAIT();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x)
    m[i] = gcmc_pick_index(k[i], n[i]);
}

__global__ void check_normals_kernel(const unsigned* w, float* out, long long n_pairs,
                                     int fast) {
  DML_GRID_WAIT();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n_pairs;
       i += (long long)gridDim.x * blockDim.x) {
    if (fast)
      normal_pair_fast(w[2 * i], w[2 * i + 1], out[2 * i], out[2 * i + 1]);
    else
      dml_normal_pair32f(w[2 * i], w[2 * i + 1], &out[2 * i], &out[2 * i + 1]);
  }
}

int k_check_normals(const unsigned* w, float* out, long long n_pairs, int fast,
                    cudaStream_t s) {
  check_normals_kernel<<<152 * 4, kBlock, 0, s>>>(w, out, n_pairs, fast);
  return 1;
}

int k_check_pick(const unsigned long long* k, const int* n, int* m, long long count, cudaStream_t s) {
  check_pick_kernel<<<152 * 4, kBlock, 0, s>>>(k, n, m, count);
  return 1;
}

// dml_get_atoms_batch: one block per replica walks its sys%alist segment in
// rounds of the block, numbering the live entries by a block scan, and
// writes each live atom's requested members at its place in the output.
__global__ void pack_atoms_kernel(Dev d, KParams p, PackOut o) {
  DML_GRID_WAIT();
  const int rep = blockIdx.x;
  const int B = d.rc[rep].base, nal = d.sc[rep].n_alist;
  const long long base = o.off[rep];
  __shared__ int s_carry;
  if (threadIdx.x == 0) s_carry = 0;
  __syncthreads();
  for (int q0 = 0; q0 < nal; q0 += blockDim.x) {
    const int q = q0 + (int)threadIdx.x;
    const int h = q < nal ? d.alist[B + q] : -1;
    int tot;
    const int pre = blk_scan_excl(h >= 0 ? 1 : 0, &tot);
    const long long i = base + s_carry + pre;
    if (h >= 0 && i < o.off[rep + 1]) {
      auto put3 = [&](double* dst, double x, double y, double z) {
        dst[3 * i] = x;
        dst[3 * i + 1] = y;
        dst[3 * i + 2] = z;
      };
      if (o.pos) {
        const double4 P = d.pos[h];
        put3(o.pos, P.x, P.y, P.z);
      }
      if (o.vel || o.acel) {
        const double4 V = d.vel[h];
        if (p.mixed) {  // FP32 velocity and acceleration in the slot (chosen form)
          const float4 v = unpack_f3(V), a = unpack_f3(make_double4(V.z, V.w, 0.0, 0.0));
          if (o.vel) put3(o.vel, v.x, v.y, v.z);
          if (o.acel) put3(o.acel, a.x, a.y, a.z);
        } else {
          if (o.vel) put3(o.vel, V.x, V.y, V.z);
          if (o.acel) {
            const double4 A = d.acel[h];
            put3(o.acel, A.x, A.y, A.z);
          }
        }
      }
      if (o.force) {
        const double4 F = d.force[h];
        put3(o.force, F.x, F.y, F.z);
      }
      if (o.pos_old) {
        const double4 O = d.pos_old[h];
        put3(o.pos_old, O.x, O.y, O.z);
      }
      if (o.old_cg) {
        const double4 O = d.old_cg[h];
        put3(o.old_cg, O.x, O.y, O.z);
      }
      if (o.epot) o.epot[i] = d.epot[h];
      if (o.z) o.z[i] = d.typ[h];
      if (o.skip) o.skip[i] = d.skip[h];
      if (o.in_ref) o.in_ref[i] = d.rank[h] >= 0 ? 1 : 0;
      if (o.in_gcmc) o.in_gcmc[i] = d.in_gcmc[h];
      if (o.id) o.id[i] = d.id[h];
    }
    __syncthreads();
    if (threadIdx.x == 0) s_carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0 && base + s_carry != o.off[rep + 1]) atomicExch(o.err, 1);
}

int k_pack_atoms(const Dev& d, const KParams& p, const PackOut& o, cudaStream_t s) {
  pack_atoms_kernel<<<d.nrep, 1024, 0, s>>>(d, p, o);
  return 1;
}

// salida (dana.F90:1143-1183) and kion (:1342-1376) for every replica.  One
// block per replica gathers its sys%alist segment in rounds of the block:
// each live atom's epot, and for a non-CG atom m (v.v) (dot_product's order,
// no contraction), go to shared memory at the atom's place in the list.  Two
// threads in different warps then add the round's terms in list order, one
// at a time, as the reference's loops do: energia over every atom, vdac over
// the non-CG ones.  Thread 0 writes the record and resets try and depo.
__global__ void __launch_bounds__(1024) salida_kernel(Dev d, KParams p, double kb,
                                                      dml_observables* out) {
  DML_GRID_WAIT();
  const int rep = blockIdx.x;
  const int B = d.rc[rep].base, nal = d.sc[rep].n_alist;
  __shared__ double s_e[1024], s_v[1024];
  __shared__ unsigned char s_m[1024];
  __shared__ double s_vdac;
  __shared__ int s_j;
  double energia = 0.0, vdac = 0.0;
  int nat = 0, j = 0;
  for (int q0 = 0; q0 < nal; q0 += blockDim.x) {
    const int q = q0 + (int)threadIdx.x;
    const int h = q < nal ? d.alist[B + q] : -1;
    int tot;
    const int k = blk_scan_excl(h >= 0 ? 1 : 0, &tot);
    if (h >= 0) {
      s_e[k] = d.epot[h];
      const int z = d.typ[h];
      s_m[k] = z != DML_Z_CG;
      if (z != DML_Z_CG) {
        const double4 V = d.vel[h];
        double vx = V.x, vy = V.y, vz = V.z;
        if (p.mixed) {  // FP32 velocity in the slot's first 16 bytes
          const float4 v = unpack_f3(V);
          vx = v.x;
          vy = v.y;
          vz = v.z;
        }
        double vd = vx * vx;
        vd = vd + vy * vy;
        vd = vd + vz * vz;
        s_v[k] = vd * p.mass[z - 1];
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int i = 0; i < tot; ++i) energia = energia + s_e[i];
      nat += tot;
    } else if (threadIdx.x == 32) {
      for (int i = 0; i < tot; ++i)
        if (s_m[i]) {
          vdac = vdac + s_v[i];
          j += 1;
        }
    }
    __syncthreads();
  }
  if (threadIdx.x == 32) {
    s_vdac = vdac;
    s_j = j;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    Scalars* sc = d.sc + rep;
    dml_observables r;
    r.step = d.g->step;
    r.energia = energia;
    r.temp = s_vdac / ((double)s_j * 3.0 * kb);
    r.rho = sc->rho;
    r.zmax = sc->zmax_frame;
    r.try_ = (int64_t)sc->try_;
    r.depo = (int64_t)sc->depo;
    r.n_atoms = nat;
    r.n_mobile = s_j;
    out[rep] = r;
    sc->try_ = 0;
    sc->depo = 0;
  }
}

int k_salida(const Dev& d, const KParams& p, double kb, dml_observables* out, cudaStream_t s) {
  salida_kernel<<<d.nrep, 1024, 0, s>>>(d, p, kb, out);
  return 1;
}

int k_check_conversions(const double* x, float* f32, double* back, long long n, cudaStream_t s) {
  check_conversions_kernel<<<152 * 4, kBlock, 0, s>>>(x, f32, back, n);
  return 1;
}

int k_load_atoms(const Dev& d, const KParams& p, const LoadIn& in, cudaStream_t s) {
  load_rep_kernel<<<152 * 8, kBlock, 0, s>>>(d);
  load_atoms_kernel<<<152 * 8, kBlock, 0, s>>>(d, p, in);
  return 2;
}
}  // namespace dml
