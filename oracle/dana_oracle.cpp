// dana_oracle.cpp - TEST INFRASTRUCTURE ONLY.
//
// A serial C++ restatement of din-mol-Li's per-step hot path, used as the
// parity oracle for the CUDA kernels and as the timed CPU baseline.  Nothing
// in the product links, imports or calls this file; only tests/, the smoke
// check and bench.py's CPU-baseline leg load the shared library built from
// it.
//
// Every routine follows the reference line by line (file:line cited beside
// each one), including its quirks: the full Verlet list with the Newton
// reaction applied twice (src/dana.F90:1125-1134), duplicate stencil cells
// when a dimension has fewer than three cells (src/Cells.F90:378-404), the
// LIFO in-cell order (src/Cells.F90:299-300), slot reuse and limbo
// (src/Groups.F90:1058-1135, src/Neighbor.F90:226-269), the single-precision
// `rsq` in gasdev (src/dana.F90:1379-1404) and the source-order floating
// point evaluation of the -O0 gfortran build (no FMA contraction; x**6 and
// x**7 by square-and-multiply).
//
// Parity pin: in RNG_NR mode this file reproduces the final frames of the
// reference's three golden runs tests/{ermak,brown,gcmc}/ref.xyz bit for bit
// (positions and element of every atom, and zmax); the CPU test suite checks
// it against the fixtures copied to tests/golden/reference/.
//
// Two random-number modes:
//   RNG_NR     the reference's own sequential ran()/gasdev() stream; with it
//              the oracle reproduces tests/{ermak,brown,gcmc}/ref.xyz.
//   RNG_PHILOX each ran()/gasdev() call site draws from the keyed Philox
//              stream of include/dml_rng.h; the GPU path is bit-exact to it.
//
// Build with -ffp-contract=off (no fused multiply-add) and without
// -ffast-math: every expression is evaluated in the reference's order.

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../include/dml.h"
#include "../include/dml_rng.h"
#include "oracle.h"

namespace {

constexpr int NUL = -1;
constexpr int LIMBO = -2;
constexpr int RNG_NR = 0;
constexpr int RNG_PHILOX = 1;

// Stencil offsets of src/Cells.F90:28-36 (cells 1-13 upper, 14-26 lower, 0 centre).
const int kMap[27][3] = {
    {0, 0, 0},   {1, 0, 0},  {1, 1, 0},   {0, 1, 0},   {-1, 1, 0},  {1, 0, -1}, {1, 1, -1},
    {0, 1, -1},  {-1, 1, -1}, {1, 0, 1},  {1, 1, 1},   {0, 1, 1},   {-1, 1, 1}, {0, 0, 1},
    {-1, 0, 0},  {-1, -1, 0}, {0, -1, 0}, {1, -1, 0},  {-1, 0, 1},  {-1, -1, 1}, {0, -1, 1},
    {1, -1, 1},  {-1, 0, -1}, {-1, -1, -1}, {0, -1, -1}, {1, -1, -1}, {0, 0, -1}};

struct Atom {
  double pos[3] = {0, 0, 0}, vel[3] = {0, 0, 0}, force[3] = {0, 0, 0}, acel[3] = {0, 0, 0};
  double pos_old[3] = {1e8, 1e8, 1e8}, old_cg[3] = {1e8, 1e8, 1e8};  // Groups.F90:300
  double epot = 0, mass = 1;
  int z = 119;
  bool skip = false;
  bool pbc[3] = {false, false, false};
  int64_t id = 0;
  int sys_slot = -1, hs_slot = -1, b_slot = -1;
  bool in_ref = false, in_gcmc = false, alive = true;
};

// igroup slot array (src/Groups.F90:179-219, 1058-1135).
struct IGroup {
  std::vector<int> a;
  int amax = 0, nat = 0, nlimbo = 0;
  bool b_limbo = false;
  // igroup_attach_atom: group_attach first increments nat, then the first
  // null slot is reused if any exists, else the index grows.
  int attach(int h, int* err) {
    nat += 1;
    int n;
    if (amax >= nat + nlimbo) {
      for (n = 0; n < amax; ++n)
        if (a[n] == NUL) break;
      if (n >= amax) {
        *err = DML_E_INDEX;  // Groups.F90:1088
        return -1;
      }
    } else {
      n = amax++;
      if ((int)a.size() < amax) a.resize(amax + 100, NUL);
    }
    a[n] = h;
    return n;
  }
  void detach(int slot) {
    a[slot] = NUL;
    nat -= 1;
  }
  // igroup_clean (Groups.F90:1036-1053)
  void clean() {
    if (!b_limbo) return;
    for (int i = 0; i < amax; ++i)
      if (a[i] == LIMBO) a[i] = NUL;
    nlimbo = 0;
    b_limbo = false;
  }
};

inline double dot3(const double* v) {
  // gfortran inlines dot_product as a left-to-right sum starting at zero.
  double s = 0.0;
  s = s + v[0] * v[0];
  s = s + v[1] * v[1];
  s = s + v[2] * v[2];
  return s;
}

// Constant integer powers r0**6, dr**6, dr**7 (dana.F90:1117-1120) as the
// reference build evaluates them: square-and-multiply from the lowest
// exponent bit, x^6 = x^2 * x^4 and x^7 = (x * x^2) * x^4.  The alternative
// power-tree chain (x^6 = x^3 * x^3) and libm pow() both fail to reproduce
// tests/ermak/ref.xyz; this chain reproduces it bit for bit.
inline double pow6(double x) {
  double x2 = x * x;
  double x4 = x2 * x2;
  return x2 * x4;
}
inline double pow7(double x) {
  double x2 = x * x;
  double x3 = x * x2;
  double x4 = x2 * x2;
  return x3 * x4;
}

// int() of a real as the x86-64 reference build computes it: truncation,
// and the integer indefinite (INT_MIN) for NaN or out-of-range values, which
// makes cgroup_sort_atom stop with "Particle out of tessellation".
inline int f2i(double x) {
  if (!(x > -2147483649.0 && x < 2147483648.0)) return INT32_MIN;
  return (int)x;
}

struct Frame {
  std::vector<double> pos;
  std::vector<int> z;
  double zmax = 0;
};

struct Sim {
  dml_params P{};
  int rng_mode = RNG_PHILOX;
  int err = 0;
  std::string errmsg;

  // NR generator state (dana.F90:1407-1428, 1379-1404)
  int32_t idum = 0, ix = -1, iy = -1;
  bool gaus_stored = false;
  double gstore = 0;

  std::vector<Atom> at;
  std::vector<int> all_list;  // sys%alist (= hs%alist = hs%b%alist order)
  std::vector<int> ref_list;  // hs%ref%alist
  std::vector<int> gcmc_list; // gcmc%alist
  std::vector<int> chunk_list;
  IGroup sys, b, hs;

  // ngroup (Neighbor.F90:32-79)
  std::vector<std::vector<int>> list;  // by hs slot
  bool listed = false;
  bool use_cells = true;  // lista / lista_atom procedure pointers
  int mnb = 10000;

  // cgroup (Cells.F90:39-84)
  bool tessellated = false;
  int ncells[3] = {1, 1, 1};
  double cell[3] = {0, 0, 0};
  std::vector<int> head;  // (0:n1+1, 0:n2+1, 0:n3+1), b slots, -1 empty
  std::vector<int> next;  // by b slot
  double rcut_b = 0;       // g%b%rcut = rc + nb_dcut (Neighbor.F90:332)

  double box[3] = {1e6, 1e6, 1e6}, one_box[3] = {1e-6, 1e-6, 1e-6};
  double z0 = 0, z1 = 0, zmax = 0, dist = 0, rho = 0, rho0 = 0;
  double zmax_frame = 0;  // zmax before the last maxz: salida's info line
  double rhomedia = 5.775329e-4, cstdev = 1.0754306e-4;  // dana.F90:445-446
  double cc0 = 0, cc1 = 0, cc2 = 0, sdr = 0, sdv = 0, crv1 = 0, crv2 = 0, skt = 0;
  std::vector<double> ranv;

  int64_t try_ = 0, depo = 0, choques = 0, choques2 = 0, choques3 = 0, nupd = 0;
  int64_t step = 0, next_id = 0, gcmc_ins = 0, gcmc_del = 0;
  int last_passes = 0;
  int max_nn = 0;
  double max_vel = 0, msd_t = 0, msd_max = 0;
  bool setup_done = false;

  // ------------------------------------------------------------------ RNG
  // ran (dana.F90:1407-1428): Marsaglia xorshift combined with Park-Miller
  // (Schrage's method); am = nearest(1.0,-1.0)/im with a single-precision
  // nearest().
  double ran() {
    const int32_t ia = 16807, im = 2147483647, iq = 127773, ir = 2836;
    const double am = (double)std::nextafter(1.0f, 0.0f) / (double)im;
    if (idum <= 0 || iy < 0) {
      iy = (888889999 ^ std::abs(idum)) | 1;
      ix = 777755555 ^ std::abs(idum);
      idum = std::abs(idum) + 1;
    }
    ix = ix ^ (int32_t)((uint32_t)ix << 13);
    ix = ix ^ (int32_t)((uint32_t)ix >> 17);
    ix = ix ^ (int32_t)((uint32_t)ix << 5);
    int32_t k = iy / iq;
    iy = ia * (iy - k * iq) - ir * k;
    if (iy < 0) iy = iy + im;
    return am * (double)((im & (ix ^ iy)) | 1);
  }
  // gasdev (dana.F90:1379-1404): polar Box-Muller, rsq kept in single
  // precision, log() of a real(4) argument is logf.
  double gasdev() {
    if (gaus_stored) {
      gaus_stored = false;
      return gstore;
    }
    double v1, v2;
    float rsq;
    for (;;) {
      v1 = 2.0 * ran() - 1.0;
      v2 = 2.0 * ran() - 1.0;
      rsq = (float)(v1 * v1 + v2 * v2);
      if ((double)rsq > 0.0 && (double)rsq < 1.0) break;
    }
    rsq = (float)std::sqrt(-2.0 * (double)logf(rsq) / (double)rsq);
    double g1 = v1 * (double)rsq;
    gstore = v2 * (double)rsq;
    gaus_stored = true;
    return g1;
  }
  double u_key(int64_t id, uint32_t stream, uint32_t sub) {
    return dml_uniform(dml_draw(P.seed, step, (uint64_t)id, stream, sub));
  }

  void fail(int code, const std::string& m) {
    if (!err) {
      err = code;
      errmsg = m;
    }
  }

  // ----------------------------------------------------------------- box
  // box_setvars (Program_Types.F90:81-95)
  void box_setvars() {
    for (int k = 0; k < 3; ++k) one_box[k] = 1.0 / box[k];
  }
  // vdistance (Groups.F90:995-1016): i - j, minimum image by idnint on the
  // dimensions where either atom is periodic.
  void vdistance(double* vd, const Atom& i, const Atom& j) const {
    for (int l = 0; l < 3; ++l) vd[l] = i.pos[l] - j.pos[l];
    for (int l = 0; l < 3; ++l)
      if (i.pbc[l] || j.pbc[l]) vd[l] = vd[l] - box[l] * (double)std::lround(vd[l] * one_box[l]);
  }
  // distance (Program_Types.F90:139-153): r2 - r1 with idnint minimum image.
  void distance(double* vd, const double* r1, const double* r2, const bool* pbc) const {
    for (int l = 0; l < 3; ++l) vd[l] = r2[l] - r1[l];
    for (int l = 0; l < 3; ++l)
      if (pbc[l]) vd[l] = vd[l] - box[l] * (double)std::lround(vd[l] * one_box[l]);
  }

  void setz(Atom& a, int z) {  // atom_setelmnt_byz (Groups.F90:615-626)
    a.z = z;
    a.mass = (z >= 1 && z <= 3) ? P.mass[z - 1] : 1.0;
  }

  // ---------------------------------------------------------------- cells
  int head_index(int c1, int c2, int c3) const {
    return (c3 * (ncells[1] + 2) + c2) * (ncells[0] + 2) + c1;
  }
  // cgroup_tessellate (Cells.F90:180-265)
  void tessellate() {
    if (tessellated) {
      bool grow_ok = true, size_ok = true;
      for (int k = 0; k < 3; ++k)
        if (!((double)(ncells[k] + 1) >= box[k] / rcut_b)) grow_ok = false;
      for (int k = 0; k < 3; ++k)
        if (!(rcut_b < box[k] / (double)ncells[k])) size_ok = false;
      if (grow_ok && size_ok) {
        for (int k = 0; k < 3; ++k) cell[k] = box[k] / (double)ncells[k];
        return;
      }
    }
    for (int k = 0; k < 3; ++k) ncells[k] = (int)(box[k] / rcut_b);
    if (ncells[0] < 4 && ncells[1] < 4 && ncells[2] < 4) return;
    for (int k = 0; k < 3; ++k) {
      if (ncells[k] < 1) {
        fail(DML_E_ARG, "box smaller than the list radius in one dimension");
        return;
      }
    }
    for (int k = 0; k < 3; ++k) cell[k] = box[k] / (double)ncells[k];
    head.assign((size_t)(ncells[0] + 2) * (ncells[1] + 2) * (ncells[2] + 2), -1);
    tessellated = true;
  }
  bool cell_of(const Atom& a, int* ci) const {
    for (int k = 0; k < 3; ++k) {
      int t = f2i(a.pos[k] / cell[k]);
      ci[k] = t == INT32_MIN ? INT32_MIN : t + 1;
    }
    return true;
  }
  // cgroup_sort_atom (Cells.F90:281-302).  silent: attach path (errors
  // switch tessellation off instead of stopping).
  void sort_atom(int i, bool silent) {
    const Atom& a = at[b.a[i]];
    int ci[3];
    cell_of(a, ci);
    bool low = ci[0] < 0 || ci[1] < 0 || ci[2] < 0;
    bool high = ci[0] > ncells[0] + 1 || ci[1] > ncells[1] + 1 || ci[2] > ncells[2] + 1;
    if (low) {
      // The reference indexes head() out of bounds here in silent mode.
      fail(DML_E_OUT_OF_TESSELLATION, "Particle out of tessellation");
      return;
    }
    if (high) {
      if (silent)
        tessellated = false;
      else
        fail(DML_E_OUT_OF_TESSELLATION, "Particle out of tessellation");
      return;
    }
    int hidx = head_index(ci[0], ci[1], ci[2]);
    next[i] = head[hidx];
    head[hidx] = i;
  }
  // cgroup_sort (Cells.F90:267-279)
  void sort_all() {
    std::fill(head.begin(), head.end(), -1);
    if ((int)next.size() < b.amax) next.resize(b.amax + 100, -1);
    for (int i = 0; i < b.amax; ++i) {
      if (b.a[i] == NUL) continue;
      sort_atom(i, false);
      if (err) return;
    }
  }
  // cgroup_unsort_atom (Cells.F90:304-352)
  void unsort_atom(int i) {
    const Atom& a = at[b.a[i]];
    int ci[3];
    cell_of(a, ci);
    for (int k = 0; k < 3; ++k)
      if (ci[k] < 0 || ci[k] > ncells[k]) {
        tessellated = false;
        return;
      }
    int hidx = head_index(ci[0], ci[1], ci[2]);
    bool removed = false;
    if (head[hidx] == i) {
      head[hidx] = next[i];
      removed = true;
    } else {
      int j = head[hidx];
      while (j >= 0) {
        int k = next[j];
        if (k == i) {
          next[j] = next[i];
          removed = true;
          break;
        }
        j = k;
      }
    }
    if (!removed) fail(DML_E_UNSORT, "Unsort cgroup particle fail");
  }
  // cell_pbc (Cells.F90:378-404) with mic = .true.: wrap in all three
  // dimensions with Fortran mod (truncating, same as C %).
  bool cell_wrap(int* r) const {
    for (int k = 0; k < 3; ++k) {
      r[k] = r[k] - 1;
      r[k] = (r[k] + ncells[k]) % ncells[k];
      r[k] = r[k] + 1;
      if (r[k] < 0 || r[k] > ncells[k] + 1) return false;
    }
    return true;
  }

  // ------------------------------------------------------ neighbour lists
  void push_neighbor(int i, int k) {
    if ((int)list[i].size() >= mnb) {
      fail(DML_E_NEIGH_OVERFLOW, "more than mnb neighbours");
      return;
    }
    list[i].push_back(k);
  }
  double list_rcut2() const {
    double r = P.rc + P.skin;
    return r * r;
  }
  // ngroup_cells_atom (Neighbor.F90:550-603)
  void cells_atom(int i) {
    list[i].clear();
    const Atom& ai = at[hs.a[i]];
    double rcut2 = list_rcut2();
    int rc[3];
    cell_of(ai, rc);
    if (rc[0] == INT32_MIN || rc[1] == INT32_MIN || rc[2] == INT32_MIN) {
      fail(DML_E_OUT_OF_TESSELLATION, "Particle out of tessellation");
      return;
    }
    for (int nabor = 0; nabor < 27; ++nabor) {
      int nc[3];
      for (int k = 0; k < 3; ++k) nc[k] = kMap[nabor][k] + rc[k];
      if (!cell_wrap(nc)) {
        fail(DML_E_OUT_OF_TESSELLATION, "stencil cell outside the head array");
        return;
      }
      int j = head[head_index(nc[0], nc[1], nc[2])];
      while (j >= 0) {
        const Atom& aj = at[b.a[j]];
        int k = aj.hs_slot;
        j = next[j];
        if (&aj == &ai) continue;
        double vd[3];
        vdistance(vd, aj, ai);
        double rd = dot3(vd);
        if (rd < rcut2) {
          push_neighbor(i, k);
          if (err) return;
        }
      }
    }
  }
  // ngroup_verlet_atom (Neighbor.F90:426-463)
  void verlet_atom(int i) {
    list[i].clear();
    const Atom& ai = at[hs.a[i]];
    double rcut2 = list_rcut2();
    for (int j = 0; j < b.amax; ++j) {
      if (b.a[j] == NUL) continue;
      const Atom& aj = at[b.a[j]];
      if (&aj == &ai) continue;
      double vd[3];
      vdistance(vd, ai, aj);
      double rd = dot3(vd);
      if (rd > rcut2) continue;
      push_neighbor(i, aj.hs_slot);
      if (err) return;
    }
  }
  void ensure_list_rows() {
    if ((int)list.size() < hs.amax) list.resize(hs.amax + 100);
  }
  // ngroup_cells / ngroup_verlet (Neighbor.F90:465-548, 358-424)
  void lista() {
    ensure_list_rows();
    for (auto& l : list) l.clear();
    hs.clean();
    for (int h : ref_list) {
      int i = at[h].hs_slot;
      if (use_cells)
        cells_atom(i);
      else
        verlet_atom(i);
      if (err) return;
    }
    max_nn = 0;
    for (int h : ref_list) max_nn = std::max(max_nn, (int)list[at[h].hs_slot].size());
    listed = true;
  }
  // update (Neighbor.F90:608-633)
  void update() {
    nupd += 1;
    for (int h : all_list)
      for (int k = 0; k < 3; ++k) at[h].pos_old[k] = at[h].pos[k];
    use_cells = tessellated;  // ngroup_setlista (Neighbor.F90:336-353)
    lista();
  }
  // do_pbc (Groups.F90:1440-1467)
  void do_pbc() {
    for (int h : all_list) {
      Atom& o = at[h];
      for (int k = 0; k < 3; ++k) {
        if (!o.pbc[k]) continue;
        if (o.pos[k] >= box[k]) {
          o.pos[k] = o.pos[k] - box[k];
          o.pos_old[k] = o.pos_old[k] - box[k];
        } else if (o.pos[k] < 0.0) {
          o.pos[k] = o.pos[k] + box[k];
          o.pos_old[k] = o.pos_old[k] + box[k];
        }
      }
    }
  }
  // test_update + inq_dispmax (Neighbor.F90:668-713, 635-666)
  int test_update() {
    do_pbc();
    tessellate();
    if (err) return 0;
    if (tessellated) sort_all();
    if (err) return 0;
    if (!listed) {
      update();
      return 1;
    }
    double d1 = 1.e-16, d2 = 1.e-16;
    for (int h : all_list) {
      const Atom& o = at[h];
      double vd[3];
      for (int k = 0; k < 3; ++k) vd[k] = o.pos[k] - o.pos_old[k];
      double rd = dot3(vd);
      if (rd > d1) {
        d2 = d1;
        d1 = rd;
      } else if (rd > d2) {
        d2 = rd;
      }
    }
    if (std::sqrt(d1) + std::sqrt(d2) > P.skin) {
      update();
      return 1;
    }
    return 0;
  }

  // ------------------------------------------------------------ integrators
  // set_ermak (dana.F90:947-971)
  void set_ermak() {
    const double h = P.h, gama = P.gamma;
    cc0 = std::exp(-h * gama);
    cc1 = (1.0 - cc0) / gama;
    cc2 = (1.0 - cc1 / h) / gama;
    sdr = std::sqrt(h / gama * (2.0 - (3.0 - 4.0 * cc0 + cc0 * cc0) / (h * gama)));
    sdv = std::sqrt(1.0 - cc0 * cc0);
    crv1 = (1.0 - cc0) * (1.0 - cc0) / (gama * sdr * sdv);
    crv2 = std::sqrt(1.0 - (crv1 * crv1));
    skt = std::sqrt(P.kb_driver * P.temp);
  }
  // atom_pbc (dana.F90:1187-1250)
  bool atom_pbc(Atom& o) {
    bool depos = false;
    for (int j = 0; j < 3; ++j) {
      if (j < 2) {
        if (o.pos[j] > box[j]) {
          o.pos[j] = o.pos[j] - box[j];
          o.pos_old[j] = o.pos_old[j] - box[j];
        }
        if (o.pos[j] < 0.0) {
          o.pos[j] = o.pos[j] + box[j];
          o.pos_old[j] = o.pos_old[j] + box[j];
        }
      } else {
        if (o.pos[j] > zmax) {
          if (P.integrator == DML_INTEGRATOR_ERMAK) {
            o.pos[2] = o.pos[2] - 2.0 * (o.pos[2] - zmax);
            o.vel[2] = -o.vel[2];
          } else {
            for (int k = 0; k < 3; ++k) o.pos[k] = o.old_cg[k];
          }
        }
      }
    }
    double msd_u = o.vel[0] * o.vel[0] * P.h * P.h;
    msd_t = msd_t + msd_u;
    if (o.pos[2] <= 0.0) {
      try_ += 1;
      double ne = rng_mode == RNG_NR ? ran() : u_key(o.id, DML_RNG_CAPTURE, 0);
      if (ne < P.prob) {
        depo += 1;
        setz(o, DML_Z_F);
        depos = true;
      }
      for (int k = 0; k < 3; ++k) o.pos[k] = o.old_cg[k];
    }
    return depos;
  }
  // ermak_a (dana.F90:974-1028)
  void ermak_a() {
    ranv.assign(ref_list.size() * 3, 0.0);
    for (size_t i = 0; i < ref_list.size(); ++i) {
      Atom& o1 = at[ref_list[i]];
      for (int k = 0; k < 3; ++k) o1.old_cg[k] = o1.pos[k];
      // Philox: (r1, r2) of x, y from draw 0 and of z from draw 1.
      double nq[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      if (rng_mode == RNG_PHILOX) {
        dml_normal_quad(dml_draw(P.seed, step, (uint64_t)o1.id, DML_RNG_ERMAK, 0), &nq[0]);
        dml_normal_quad(dml_draw(P.seed, step, (uint64_t)o1.id, DML_RNG_ERMAK, 1), &nq[4]);
      }
      for (int j = 0; j < 3; ++j) {
        double r1, r2 = 0;
        if (rng_mode == RNG_NR) {
          r1 = gasdev();
        } else {
          r1 = nq[2 * j];
          r2 = nq[2 * j + 1];
        }
        double ranr = skt / std::sqrt(o1.mass) * sdr * r1;
        o1.pos[j] = o1.pos[j] + cc1 * o1.vel[j] + cc2 * P.h * o1.acel[j] + ranr;
        if (rng_mode == RNG_NR) r2 = gasdev();
        ranv[i * 3 + j] = skt / std::sqrt(o1.mass) * sdv * (crv1 * r1 + crv2 * r2);
      }
      bool depos = atom_pbc(o1);
      if (depos) continue;
      o1.skip = false;
    }
  }
  // ermak_b (dana.F90:1031-1052)
  void ermak_b() {
    for (size_t i = 0; i < ref_list.size(); ++i) {
      Atom& o1 = at[ref_list[i]];
      if (o1.z == DML_Z_CG) continue;
      for (int l = 0; l < 3; ++l)
        o1.vel[l] = cc0 * o1.vel[l] + (cc1 - cc2) * o1.acel[l] + cc2 * o1.force[l] / o1.mass + ranv[i * 3 + l];
      for (int l = 0; l < 3; ++l) o1.acel[l] = o1.force[l] / o1.mass;
    }
  }
  // cbrownian_hs (dana.F90:798-846)
  void brownian() {
    for (int h : ref_list) {
      Atom& o1 = at[h];
      for (int k = 0; k < 3; ++k) o1.old_cg[k] = o1.pos[k];
      double dif = o1.pos[2] > P.dif_switch_z ? P.dif_sc : P.dif_sei;
      double fac1 = std::sqrt(2.0 * dif * P.h);
      double nrm[4] = {0, 0, 0, 0};
      if (rng_mode == RNG_PHILOX)
        dml_normal_quad(dml_draw(P.seed, step, (uint64_t)o1.id, DML_RNG_BROWN, 0), nrm);
      for (int j = 0; j < 3; ++j) {
        double r1 = rng_mode == RNG_NR ? gasdev() : nrm[j];
        double posold = o1.pos[j];
        o1.pos[j] = posold + r1 * fac1;
        o1.vel[j] = (o1.pos[j] - posold) / P.h;
      }
      bool depos = atom_pbc(o1);
      if (depos) continue;
      max_vel = std::max(max_vel, dot3(o1.vel));
      o1.skip = false;
    }
  }
  // fuerza (dana.F90:1055-1139)
  void fuerza() {
    for (int h : ref_list) {
      Atom& o1 = at[h];
      for (int l = 0; l < 3; ++l) o1.force[l] = 0.0;
      o1.epot = 0.0;
    }
    for (int h : ref_list) {
      Atom& o1 = at[h];
      int i = o1.hs_slot;
      int k = o1.z;
      for (int j : list[i]) {
        if (hs.b_limbo && hs.a[j] == LIMBO) continue;
        Atom& o2 = at[hs.a[j]];
        int m = o2.z;
        double vd[3];
        for (int l = 0; l < 3; ++l) vd[l] = o1.pos[l] - o2.pos[l];
        for (int l = 0; l < 2; ++l) {
          if (vd[l] > box[l] * .5) {
            vd[l] = vd[l] - box[l];
          } else if (vd[l] < -box[l] * .5) {
            vd[l] = vd[l] + box[l];
          }
        }
        if (o2.z == DML_Z_CG && o1.z == DML_Z_CG) continue;
        double dr = dot3(vd);
        double r0km = P.r0[k - 1][m - 1], epskm = P.eps[k - 1][m - 1];
        if (dr > r0km * r0km) continue;
        dr = std::sqrt(dr);
        double bb = pow6(r0km);
        double c = epskm * 12.0 * bb;
        c = c / pow7(dr);
        bb = bb / pow6(dr);
        double aux = c * (bb - 1.0);
        for (int l = 0; l < 3; ++l) o1.force[l] = o1.force[l] + aux * vd[l] / dr;
        for (int l = 0; l < 3; ++l) o2.force[l] = o2.force[l] - aux * vd[l] / dr;
        aux = epskm * bb * (bb - 2.0);
        aux = aux + epskm;
        o1.epot = o1.epot + aux * .5;
        o2.epot = o2.epot + aux * .5;
      }
    }
  }
  // overlap_moveback (dana.F90:849-943); the recursion is a loop over passes.
  void overlap_moveback() {
    const double rcut2 = P.rc * P.rc;  // ngroup_setrc (Neighbor.F90:330)
    int maxp = P.max_passes > 0 ? P.max_passes : 64;
    int pass = 0;
    int64_t c_after_first = -1;
    bool again;
    do {
      pass += 1;
      if (pass > maxp) {
        fail(DML_E_OVERLAP_PASSES, "overlap_moveback exceeded the pass cap");
        return;
      }
      again = false;
      for (int h : ref_list) {
        Atom& o1 = at[h];
        if (o1.skip) continue;
        o1.skip = true;
        int i = o1.hs_slot;
        for (int j : list[i]) {
          if (hs.b_limbo && hs.a[j] == LIMBO) continue;
          Atom& o2 = at[hs.a[j]];
          double vd[3];
          vdistance(vd, o1, o2);
          double dr = dot3(vd);
          if (dr > rcut2) continue;
          if (o2.z == DML_Z_CG) {
            try_ += 1;
            double ne = rng_mode == RNG_NR ? ran() : u_key(o1.id, DML_RNG_OVERLAP, (uint32_t)pass);
            if (ne < P.prob) {
              depo += 1;
              setz(o1, DML_Z_F);
              if (o1.pos[2] > z0) {
                fail(DML_E_DENDRITE, "deposit above z0");
                return;
              }
            } else {
              for (int l = 0; l < 3; ++l) o1.pos[l] = o1.old_cg[l];
              o1.skip = false;
            }
            break;
          }
          if (P.reservoir == DML_RESERVOIR_PISTON) {
            bool o2_old = o2.pos[0] == o2.old_cg[0] && o2.pos[1] == o2.old_cg[1] && o2.pos[2] == o2.old_cg[2];
            bool o1_old = o1.pos[0] == o1.old_cg[0] && o1.pos[1] == o1.old_cg[1] && o1.pos[2] == o1.old_cg[2];
            if (o2_old && o1_old) {
              choques3 += 1;
              continue;
            }
          }
          for (int l = 0; l < 3; ++l) {
            o2.pos[l] = o2.old_cg[l];
            o2.acel[l] = 0.0;
            o2.vel[l] = 0.0;
          }
          o2.skip = false;
          choques += 1;
          again = true;
        }
      }
      if (pass == 1) c_after_first = choques;
    } while (again);
    last_passes = pass;
    choques2 = std::max(choques2, choques - c_after_first);
  }
  // Capture commit (dana.F90:226-236)
  int capture_commit() {
    int nnew = 0;
    std::vector<int> keep;
    keep.reserve(ref_list.size());
    for (int h : ref_list) {
      Atom& o1 = at[h];
      if (o1.z != DML_Z_F) {
        keep.push_back(h);
        continue;
      }
      setz(o1, DML_Z_CG);
      o1.in_ref = false;
      nnew += 1;
      if (P.reservoir == DML_RESERVOIR_GCMC && o1.in_gcmc) {
        o1.in_gcmc = false;
        gcmc_list.erase(std::find(gcmc_list.begin(), gcmc_list.end(), h));
      }
    }
    ref_list.swap(keep);
    return nnew;
  }
  // calc_rho (dana.F90:521-549)
  void calc_rho() {
    double zt = P.reservoir == DML_RESERVOIR_CHUNKS ? z1 : zmax;
    int g = 0;
    for (int h : all_list)
      if (at[h].pos[2] > z0 && at[h].pos[2] < zt) g += 1;
    double vol = box[0] * box[1] * (zt - z0);
    rho = (double)g / vol;
  }
  // maxz (dana.F90:776-794)
  void maxz() {
    zmax_frame = zmax;
    double lohi = ((P.h / P.tau) * ((rho0 - rho) / rho));
    for (int h : all_list) {
      Atom& pa = at[h];
      if (pa.pos[2] > z0) pa.pos[2] = pa.pos[2] - lohi * (pa.pos[2] - z0);
    }
    zmax = zmax - lohi * (zmax - z0);
  }

  // --------------------------------------------------------- structure edits
  int new_atom() {
    Atom a;
    a.id = next_id++;
    at.push_back(a);
    return (int)at.size() - 1;
  }
  // Attach to sys, hs%ref, hs%b, hs in group-id order (Groups.F90:730-766,
  // 1058-1100; Cells.F90:105-144; Neighbor.F90:173-224).
  void attach_sys(int h) {
    at[h].sys_slot = sys.attach(h, &err);
    all_list.push_back(h);
  }
  void attach_ref(int h) {
    at[h].in_ref = true;
    ref_list.push_back(h);
  }
  void attach_b(int h, bool sort_now) {
    int i = b.attach(h, &err);
    at[h].b_slot = i;
    if ((int)next.size() < b.amax) next.resize(b.amax + 100, -1);
    if (tessellated && sort_now) sort_atom(i, true);
  }
  void attach_hs(int h) {
    int i = hs.attach(h, &err);
    if (err) return;
    at[h].hs_slot = i;
    ensure_list_rows();
    if (listed) ngroup_sort_atom(i);
  }
  // ngroup_sort_atom (Neighbor.F90:271-318)
  void ngroup_sort_atom(int i) {
    list[i].clear();
    Atom& a = at[hs.a[i]];
    if (a.in_ref) {
      if (use_cells)
        cells_atom(i);
      else
        verlet_atom(i);
      if (err) return;
    }
    double rcut2 = list_rcut2();
    for (int h : ref_list) {
      Atom& aj = at[h];
      int j = aj.hs_slot;
      if (&aj == &a) continue;
      double vd[3];
      vdistance(vd, a, aj);
      double rd = dot3(vd);
      if (rd > rcut2) continue;
      push_neighbor(j, i);
      if (err) return;
    }
  }
  // atom_destroy (Groups.F90:433-467): detach LIFO by group id:
  // gcmc, hs (-> ref, b), sys.
  void destroy_atom(int h) {
    Atom& o = at[h];
    if (o.in_gcmc) {
      gcmc_list.erase(std::find(gcmc_list.begin(), gcmc_list.end(), h));
      o.in_gcmc = false;
    }
    // ngroup_detach_atom (Neighbor.F90:226-269)
    int i = o.hs_slot;
    if (listed) list[i].clear();
    if (o.in_ref) {
      ref_list.erase(std::find(ref_list.begin(), ref_list.end(), h));
      o.in_ref = false;
    }
    if (tessellated && o.b_slot >= 0) unsort_atom(o.b_slot);
    if (err) return;
    b.detach(o.b_slot);
    o.b_slot = -1;
    hs.detach(i);
    if (listed) {
      hs.a[i] = LIMBO;
      hs.nlimbo += 1;
      hs.b_limbo = true;
    }
    o.hs_slot = -1;
    sys.detach(o.sys_slot);
    o.sys_slot = -1;
    all_list.erase(std::find(all_list.begin(), all_list.end(), h));
    o.alive = false;
  }
  // atom_asign (Groups.F90:484-502)
  void atom_asign(Atom& a1, const Atom& a2) {
    for (int k = 0; k < 3; ++k) {
      a1.pos[k] = a2.pos[k];
      a1.vel[k] = a2.vel[k];
      a1.force[k] = a2.force[k];
      a1.acel[k] = a2.acel[k];
      a1.pbc[k] = a2.pbc[k];
      a1.pos_old[k] = a2.pos_old[k];
    }
    setz(a1, a2.z);
    a1.epot = a2.epot;
  }

  // gcmc_run (dana.F90:590-713)
  void gcmc_run() {
    const double rc = P.rc;
    double v = box[0] * box[1] * (zmax - z0);
    int n = 0;
    for (int h : gcmc_list) {
      const Atom& o = at[h];
      if (o.pos[2] < z0 || o.pos[2] > zmax) continue;
      n = n + 1;
    }
    for (int t = 1; t <= P.nadj; ++t) {
      if (gcmc_list.empty()) {
        fail(DML_E_NO_PARTICLES, "No more particles");
        return;
      }
      int href = gcmc_list[0];
      double beta = std::sqrt(P.kb_module * P.temp / at[href].mass);
      dml_u4 w0{}, w1{}, w2{};
      if (rng_mode == RNG_PHILOX) {
        w0 = dml_draw(P.seed, step, (uint64_t)t, DML_RNG_GCMC, 0);
        w1 = dml_draw(P.seed, step, (uint64_t)t, DML_RNG_GCMC, 1);
        w2 = dml_draw(P.seed, step, (uint64_t)t, DML_RNG_GCMC, 2);
      }
      double coin = rng_mode == RNG_NR ? ran() : dml_u53(w0.w[0], w0.w[1]);
      if (coin < 0.5) {
        double uacc = rng_mode == RNG_NR ? ran() : dml_u53(w0.w[2], w0.w[3]);
        if (P.act * v / (double)(n + 1) < uacc) continue;
        double r[3];
        if (rng_mode == RNG_NR) {
          r[0] = ran() * box[0];
          r[1] = ran() * box[1];
          r[2] = ran() * (zmax - z0) + z0;
        } else {
          r[0] = dml_u53(w1.w[0], w1.w[1]) * box[0];
          r[1] = dml_u53(w1.w[2], w1.w[3]) * box[1];
          r[2] = dml_u53(w2.w[0], w2.w[1]) * (zmax - z0) + z0;
        }
        bool overlap = false;
        for (int h : gcmc_list) {
          const Atom& o = at[h];
          double vd[3];
          distance(vd, o.pos, r, o.pbc);
          double dr = dot3(vd);
          if (dr < rc * rc) {
            overlap = true;
            break;
          }
        }
        if (overlap) continue;
        int hlast = gcmc_list.back();
        n = n + 1;
        int ho = new_atom();
        Atom& o = at[ho];
        atom_asign(o, at[href]);
        for (int k = 0; k < 3; ++k) {
          o.pos[k] = r[k];
          o.pos_old[k] = r[k];
        }
        // Maxwell velocity written to the last atom of the list (dana.F90:666-668).
        if (rng_mode == RNG_NR) {
          for (int j = 0; j < 3; ++j) at[hlast].vel[j] = beta * gasdev();
        } else {
          double nv[4];
          dml_normal_quad(dml_draw(P.seed, step, (uint64_t)t, DML_RNG_GCMC_VEL, 0), nv);
          for (int j = 0; j < 3; ++j) at[hlast].vel[j] = beta * nv[j];
        }
        // Same groups as the template, in group-id order: sys, ref, b, hs, gcmc.
        attach_sys(ho);
        attach_ref(ho);
        attach_b(ho, true);
        if (err) return;
        attach_hs(ho);
        if (err) return;
        at[ho].in_gcmc = true;
        gcmc_list.push_back(ho);
        gcmc_ins += 1;
      } else {
        double uacc = rng_mode == RNG_NR ? ran() : dml_u53(w0.w[2], w0.w[3]);
        if ((double)n / (v * P.act) < uacc) continue;
        double upick = rng_mode == RNG_NR ? ran() : dml_u53(w2.w[2], w2.w[3]);
        int m = (int)std::floor(upick * (double)n) + 1;
        if (m > n) m = n;
        int hsel = -1;
        for (int h : gcmc_list) {
          const Atom& o = at[h];
          hsel = h;
          if (o.pos[2] < z0) continue;
          if (o.pos[2] > zmax) continue;
          m = m - 1;
          if (m == 0) break;
        }
        if (m > 0) {
          fail(DML_E_CHOSEN_MISSING, "Chosen particle does not exists");
          return;
        }
        n = n - 1;
        destroy_atom(hsel);
        if (err) return;
        gcmc_del += 1;
      }
    }
  }

  // bloques (dana.F90:716-773): chunk reservoir.
  void bloques() {
    double drho = rho - rhomedia;
    if (std::fabs(drho) < (rhomedia * (double)0.186f)) return;
    z0 = z0 + dist;
    z1 = z1 + dist;
    zmax = zmax + dist;
    zmax_frame = zmax;  // salida's info line reports the new top
    listed = false;
    std::vector<int> chunk = chunk_list;
    for (int h1 : chunk) {
      int h2 = new_atom();
      attach_sys(h2);
      // The reference sorts the zero-initialised atom into cell (1,1,1) here;
      // the full re-sort in the test_update below overwrites that chain.
      attach_b(h2, false);
      attach_ref(h2);
      attach_hs(h2);
      if (err) return;
      Atom& o1 = at[h1];
      Atom& o2 = at[h2];
      atom_asign(o2, o1);
      for (int k = 0; k < 3; ++k) o2.pbc[k] = o1.pbc[k];
      o1.pos[2] = o1.pos[2] + dist;
      o1.pos_old[2] = o1.pos_old[2] + dist;
    }
    box[2] = zmax;
    box_setvars();
    test_update();
  }

  // ---------------------------------------------------------- step driver
  // Loop body of dana.F90:173-247 (up to and including the reservoirs,
  // before salida).
  void step_body() {
    step += 1;
    if (P.integrator == DML_INTEGRATOR_ERMAK) {
      ermak_a();
      fuerza();
      ermak_b();
    } else {
      brownian();
    }
    test_update();
    if (err) return;
    overlap_moveback();
    if (err) return;
    test_update();
    if (err) return;
    if (!ref_list.empty()) msd_t = msd_t / (double)ref_list.size();
    msd_max = std::max(msd_max, msd_t);
    capture_commit();
    if (P.reservoir == DML_RESERVOIR_GCMC) gcmc_run();
    if (err) return;
    calc_rho();
    if (P.reservoir == DML_RESERVOIR_CHUNKS) bloques();
  }
  // dana.F90:261 (after salida)
  void step_tail() {
    if (P.reservoir == DML_RESERVOIR_PISTON) maxz();
  }

  // Start-up after the atoms are loaded (dana.F90:127-146).
  void setup() {
    box_setvars();
    rcut_b = P.rc + P.skin;
    if (P.integrator == DML_INTEGRATOR_ERMAK) set_ermak();
    test_update();
    if (err) return;
    if (P.integrator == DML_INTEGRATOR_ERMAK) fuerza();
    calc_rho();
    rho0 = rho;
    setup_done = true;
  }

  // salida (dana.F90:1143-1183): energia, the sum of epot over sys%alist
  // (:1155-1159), and kion(sys, temp) (:1342-1376), each adding one term at a
  // time in list order; try and depo are written, then reset (:1168-1174).
  dml_observables salida() {
    dml_observables r;
    std::memset(&r, 0, sizeof r);
    double energia = 0.0;
    for (int h : all_list) energia = energia + at[h].epot;
    double vdac = 0.0;
    int j = 0;
    for (int h : all_list) {
      const Atom& o1 = at[h];
      if (o1.z == DML_Z_CG) continue;  // kion skips metallic Li
      j = j + 1;
      double vd = 0.0;  // dot_product(vel, vel)
      for (int l = 0; l < 3; ++l) vd = vd + o1.vel[l] * o1.vel[l];
      vd = vd * o1.mass;
      vdac = vdac + vd;
    }
    r.step = step;
    r.energia = energia;
    r.temp = vdac / ((double)j * 3.0 * P.kb_driver);
    r.rho = rho;
    r.zmax = zmax_frame;
    r.try_ = try_;
    r.depo = depo;
    r.n_atoms = (int32_t)all_list.size();
    r.n_mobile = j;
    try_ = 0;
    depo = 0;
    return r;
  }

  Frame frame() const {
    Frame f;
    for (int h : all_list) {
      for (int k = 0; k < 3; ++k) f.pos.push_back(at[h].pos[k]);
      f.z.push_back(at[h].z);
    }
    f.zmax = zmax;
    return f;
  }
};

// --------------------------------------------------------------- NR harness
// Reproduces the reference executable on a tests/<case>/ directory:
// entrada (dana.F90:309-327), pos_inic (:330-396), config_run (:399-427),
// config_inic (:430-517), config_chunk (:552-587) and the step loop; keeps
// the last frame that salida (:1143-1183) would write.
struct RefCase {
  int32_t idum;
  double prob, h;
  int nst, nwr;
  double xi, yi, dist, z0, zmax, dif_sc, dif_sei, nb_dcut;
  bool integrador;
  std::string reservoir;
  double act = 0;
  int nadj = 0;
};

std::string first_token(const std::string& line) {
  std::istringstream is(line);
  std::string t;
  is >> t;
  return t;
}

bool read_case(const std::string& dir, RefCase* c) {
  std::ifstream f(dir + "/entrada.ini");
  if (!f) return false;
  std::string l[13];
  for (int i = 0; i < 13; ++i)
    if (!std::getline(f, l[i])) return false;
  c->idum = (int32_t)std::stol(first_token(l[0]));
  c->prob = std::stod(first_token(l[1]));
  c->h = std::stod(first_token(l[2]));
  c->nst = std::stoi(first_token(l[3]));
  c->nwr = std::stoi(first_token(l[4]));
  c->xi = std::stod(first_token(l[5]));
  c->yi = std::stod(first_token(l[6]));
  c->dist = std::stod(first_token(l[7]));
  c->z0 = std::stod(first_token(l[8]));
  c->zmax = std::stod(first_token(l[9]));
  c->dif_sc = std::stod(first_token(l[10]));
  c->dif_sei = std::stod(first_token(l[11]));
  c->nb_dcut = std::stod(first_token(l[12]));
  std::ifstream m(dir + "/movedor.ini");
  if (!m) return false;
  std::string a;
  std::getline(m, a);
  std::string t = first_token(a);
  for (auto& ch : t) ch = (char)std::tolower((unsigned char)ch);
  c->integrador = t.find(".true.") != std::string::npos || t == "t" || t == ".t.";
  std::getline(m, a);
  c->reservoir = first_token(a);
  if (c->reservoir == "gcmc") {
    std::getline(m, a);
    std::istringstream is(a);
    is >> c->act >> c->nadj;
  }
  return true;
}

// f25.12 write then read back (dana.F90:391, 463).
double f25_12(double x) {
  char buf[64];
  std::snprintf(buf, sizeof buf, "%25.12f", x);
  return std::strtod(buf, nullptr);
}

}  // namespace

// ============================================================== C interface

struct orc_sim {
  Sim s;
  std::vector<Frame> frames;
};

extern "C" {

orc_sim* orc_create(const dml_params* p, int32_t rng_mode, int32_t idum) {
  orc_sim* o = new orc_sim();
  o->s.P = *p;
  o->s.rng_mode = rng_mode;
  o->s.idum = idum;
  o->s.mnb = p->mnb > 0 ? p->mnb : 10000;
  for (int k = 0; k < 3; ++k) o->s.box[k] = p->box[k];
  o->s.z0 = p->z0;
  o->s.z1 = p->z1;
  o->s.zmax = p->zmax;
  o->s.zmax_frame = p->zmax;
  o->s.rcut_b = p->rc + p->skin;
  o->s.box_setvars();
  return o;
}

void orc_destroy(orc_sim* o) { delete o; }

int orc_set_atoms(orc_sim* o, const dml_atoms* a) {
  Sim& s = o->s;
  for (int i = 0; i < a->n; ++i) {
    int h = s.new_atom();
    Atom& x = s.at[h];
    for (int k = 0; k < 3; ++k) {
      x.pos[k] = a->pos[3 * i + k];
      x.vel[k] = a->vel ? a->vel[3 * i + k] : 0.0;
      x.acel[k] = a->acel ? a->acel[3 * i + k] : 0.0;
      x.force[k] = a->force ? a->force[3 * i + k] : 0.0;
      x.pos_old[k] = a->pos_old ? a->pos_old[3 * i + k] : x.pos[k];
      x.old_cg[k] = a->old_cg ? a->old_cg[3 * i + k] : 1e8;
    }
    x.epot = a->epot ? a->epot[i] : 0.0;
    s.setz(x, a->z[i]);
    x.skip = a->skip ? a->skip[i] != 0 : false;
    x.pbc[0] = x.pbc[1] = true;
    x.pbc[2] = false;
    if (a->id) {
      x.id = a->id[i];
      s.next_id = std::max(s.next_id, x.id + 1);
    }
    bool in_ref = a->in_ref ? a->in_ref[i] != 0 : (x.z != DML_Z_CG);
    // config_inic attach order (dana.F90:468-480)
    s.attach_sys(h);
    if (in_ref) s.attach_ref(h);
    s.attach_b(h, false);
    s.attach_hs(h);
    if (s.err) return s.err;
  }
  // gcmc attach loop (dana.F90:130-137): all z==1 atoms in sys order.
  if (s.P.reservoir == DML_RESERVOIR_GCMC) {
    for (int i = 0; i < a->n; ++i) {
      int h = s.all_list[i];
      bool g = a->in_gcmc ? a->in_gcmc[i] != 0 : (s.at[h].z == DML_Z_LI);
      if (g) {
        s.at[h].in_gcmc = true;
        s.gcmc_list.push_back(h);
      }
    }
  }
  return s.err;
}

int orc_setup(orc_sim* o) {
  o->s.setup();
  return o->s.err;
}

int orc_step(orc_sim* o, int64_t nsteps) {
  for (int64_t i = 0; i < nsteps; ++i) {
    o->s.step_body();
    if (o->s.err) return o->s.err;
    o->s.step_tail();
  }
  return o->s.err;
}

int orc_test_update(orc_sim* o, int32_t* rebuilt) {
  int r = o->s.test_update();
  if (rebuilt) *rebuilt = r;
  return o->s.err;
}
int orc_force(orc_sim* o) {
  o->s.fuerza();
  return o->s.err;
}
int orc_ermak_a(orc_sim* o, int64_t step) {
  o->s.step = step;
  o->s.ermak_a();
  return o->s.err;
}
int orc_ermak_b(orc_sim* o) {
  o->s.ermak_b();
  return o->s.err;
}
int orc_brownian(orc_sim* o, int64_t step) {
  o->s.step = step;
  o->s.brownian();
  return o->s.err;
}
int orc_overlap_moveback(orc_sim* o, int64_t step) {
  o->s.step = step;
  o->s.overlap_moveback();
  return o->s.err;
}
int orc_capture_commit(orc_sim* o, int32_t* n_new) {
  int n = o->s.capture_commit();
  if (n_new) *n_new = n;
  return o->s.err;
}
int orc_gcmc(orc_sim* o, int64_t step) {
  o->s.step = step;
  o->s.gcmc_run();
  return o->s.err;
}
// config_chunk (dana.F90:552-587) from arrays instead of chunk.xyz: n
// template atoms at pos (as the file gives them) with elements z, raised by
// zmax (pos_old by twice zmax, as the reference writes it), outside every
// group; dist is the chunk height (entrada.ini's dist plus rc, :437-441).
int orc_set_chunk(orc_sim* o, int32_t n, const double* pos, const int32_t* z, double dist) {
  Sim& s = o->s;
  if (n <= 0 || !pos || !z) return DML_E_ARG;
  s.dist = dist;
  for (int j = 0; j < n; ++j) {
    const int h = s.new_atom();
    Atom& a = s.at[h];
    for (int k = 0; k < 3; ++k) a.pos[k] = pos[3 * j + k];
    s.setz(a, z[j]);
    for (int k = 0; k < 3; ++k) {
      a.force[k] = 0.0;
      a.pos_old[k] = a.pos[k];
    }
    a.pos[2] = a.pos[2] + s.zmax;
    a.pos_old[2] = a.pos[2] + s.zmax;
    a.pbc[0] = a.pbc[1] = true;
    a.pbc[2] = false;
    s.chunk_list.push_back(h);
  }
  return 0;
}

// bloques (dana.F90:716-773) on its own.
int orc_bloques(orc_sim* o) {
  o->s.bloques();
  return o->s.err;
}

int orc_calc_rho(orc_sim* o, double* rho) {
  o->s.calc_rho();
  if (rho) *rho = o->s.rho;
  return o->s.err;
}
int orc_piston(orc_sim* o) {
  o->s.maxz();
  return o->s.err;
}

int orc_get_atoms(orc_sim* o, dml_atoms* a) {
  const Sim& s = o->s;
  int n = (int)s.all_list.size();
  if (a->n < n) return DML_E_ARG;
  a->n = n;
  for (int i = 0; i < n; ++i) {
    const Atom& x = s.at[s.all_list[i]];
    for (int k = 0; k < 3; ++k) {
      if (a->pos) a->pos[3 * i + k] = x.pos[k];
      if (a->vel) a->vel[3 * i + k] = x.vel[k];
      if (a->acel) a->acel[3 * i + k] = x.acel[k];
      if (a->force) a->force[3 * i + k] = x.force[k];
      if (a->pos_old) a->pos_old[3 * i + k] = x.pos_old[k];
      if (a->old_cg) a->old_cg[3 * i + k] = x.old_cg[k];
    }
    if (a->epot) a->epot[i] = x.epot;
    if (a->z) a->z[i] = x.z;
    if (a->skip) a->skip[i] = x.skip ? 1 : 0;
    if (a->in_ref) a->in_ref[i] = x.in_ref ? 1 : 0;
    if (a->in_gcmc) a->in_gcmc[i] = x.in_gcmc ? 1 : 0;
    if (a->id) a->id[i] = x.id;
  }
  return 0;
}

int orc_get_neighbors(orc_sim* o, int32_t* n_ref, int32_t* nn, int32_t* list, int32_t ld) {
  const Sim& s = o->s;
  // hs slot -> sys%alist position
  std::vector<int> pos_of(s.hs.amax + 1, -1);
  for (size_t i = 0; i < s.all_list.size(); ++i) {
    int sl = s.at[s.all_list[i]].hs_slot;
    if (sl >= 0) pos_of[sl] = (int)i;
  }
  *n_ref = (int32_t)s.ref_list.size();
  for (size_t k = 0; k < s.ref_list.size(); ++k) {
    const Atom& x = s.at[s.ref_list[k]];
    const std::vector<int>& row = s.list[x.hs_slot];
    nn[k] = (int32_t)row.size();
    if ((int)row.size() > ld) return DML_E_ARG;
    for (size_t jj = 0; jj < row.size(); ++jj) {
      int sl = row[jj];
      list[k * (size_t)ld + jj] = (s.hs.a[sl] == LIMBO) ? -1 : pos_of[sl];
    }
  }
  return 0;
}

int orc_get_counters(orc_sim* o, dml_counters* c) {
  const Sim& s = o->s;
  std::memset(c, 0, sizeof *c);
  c->try_ = s.try_;
  c->depo = s.depo;
  c->choques = s.choques;
  c->choques3 = s.choques3;
  c->nupd = s.nupd;
  c->step = s.step;
  c->gcmc_ins = s.gcmc_ins;
  c->gcmc_del = s.gcmc_del;
  c->n_atoms = (int32_t)s.all_list.size();
  c->n_ref = (int32_t)s.ref_list.size();
  c->max_nn = s.max_nn;
  c->passes = s.last_passes;
  c->zmax = s.zmax;
  c->z0 = s.z0;
  c->rho = s.rho;
  c->rho0 = s.rho0;
  return 0;
}

int orc_reset_counters(orc_sim* o) {
  o->s.try_ = 0;
  o->s.depo = 0;
  return 0;
}

int orc_salida(orc_sim* o, dml_observables* out) {
  *out = o->s.salida();
  return 0;
}

const char* orc_errmsg(orc_sim* o) { return o->s.errmsg.c_str(); }

void orc_set_step(orc_sim* o, int64_t step) { o->s.step = step; }

// Runs one reference test directory in NR mode and returns the last frame
// that salida would have written.  max_n is the capacity of pos_out/z_out.
int orc_run_reference_case(const char* dir, int32_t max_n, int32_t* n_out, double* pos_out,
                           int32_t* z_out, double* zmax_out, int64_t* counters_out) {
  RefCase c;
  if (!read_case(dir, &c)) return DML_E_ARG;
  dml_params p;
  dml_params_default_oracle(&p);
  p.prob = c.prob;
  p.h = c.h;
  p.skin = c.nb_dcut;
  p.z0 = c.z0;
  p.zmax = c.zmax;
  p.dif_sc = c.dif_sc;
  p.dif_sei = c.dif_sei;
  p.integrator = c.integrador ? DML_INTEGRATOR_ERMAK : DML_INTEGRATOR_BROWNIAN;
  if (c.reservoir == "piston")
    p.reservoir = DML_RESERVOIR_PISTON;
  else if (c.reservoir == "chunks")
    p.reservoir = DML_RESERVOIR_CHUNKS;
  else if (c.reservoir == "gcmc")
    p.reservoir = DML_RESERVOIR_GCMC;
  else
    return DML_E_RESERVOIR;
  p.act = c.act;
  p.nadj = c.nadj;
  p.box[0] = c.xi;
  p.box[1] = c.yi;
  p.box[2] = c.zmax;  // pos_inic sets the box from the entrada zmax (dana.F90:342-346)
  p.mnb = 10000;
  orc_sim* o = orc_create(&p, RNG_NR, c.idum);
  Sim& s = o->s;
  s.dist = c.dist;

  // pos_inic (dana.F90:330-396)
  {
    s.box_setvars();
    double alto = c.zmax - 0.0;
    int n = (int)(1.0 * c.xi * c.yi * alto * (double)6.022e-4f);
    std::vector<double> r((size_t)n * 3);
    const bool pbc[3] = {true, true, false};
    const double r0 = 3.2;
    for (int i = 0; i < n; ++i) {
      int k;
      for (k = 1; k <= 10000; ++k) {
        r[3 * i + 0] = s.ran() * c.xi;
        r[3 * i + 1] = s.ran() * c.yi;
        r[3 * i + 2] = (s.ran() * alto) + 0.0;
        bool ok = true;
        for (int j = 0; j < i; ++j) {
          double vd[3];
          s.distance(vd, &r[3 * j], &r[3 * i], pbc);
          double dif2 = dot3(vd);
          if (dif2 < r0 * r0) {
            ok = false;
            break;
          }
        }
        if (ok) break;
      }
      if (k == 10001) {
        orc_destroy(o);
        return DML_E_RSA;
      }
    }
    // config_inic (dana.F90:430-517): chunk sensor sizes first.
    if (p.reservoir == DML_RESERVOIR_CHUNKS) {
      s.dist = s.dist + p.rc;  // dist + hs%rcut
      s.z1 = s.z0 + s.dist;
      s.zmax = s.z1 + s.dist;
    }
    for (int i = 0; i < n; ++i) {
      int h = s.new_atom();
      Atom& x = s.at[h];
      for (int k = 0; k < 3; ++k) x.pos[k] = f25_12(r[3 * i + k]);
      s.setz(x, DML_Z_LI);
      for (int k = 0; k < 3; ++k) {
        x.force[k] = 0.0;
        x.pos_old[k] = x.pos[k];
      }
      x.pbc[0] = x.pbc[1] = true;
      x.pbc[2] = false;
      s.attach_sys(h);
      s.attach_ref(h);
      s.attach_b(h, false);
      s.attach_hs(h);
    }
  }
  if (p.reservoir == DML_RESERVOIR_GCMC) {
    for (int h : s.all_list)
      if (s.at[h].z == DML_Z_LI) {
        s.at[h].in_gcmc = true;
        s.gcmc_list.push_back(h);
      }
  }
  // Start-up (dana.F90:140-146)
  if (p.integrator == DML_INTEGRATOR_ERMAK) s.set_ermak();
  s.test_update();
  if (p.integrator == DML_INTEGRATOR_ERMAK) s.fuerza();
  s.calc_rho();
  s.rho0 = s.rho;
  // config_chunk (dana.F90:552-587)
  if (p.reservoir == DML_RESERVOIR_CHUNKS) {
    std::ifstream f(std::string(dir) + "/chunk.xyz");
    if (!f) {
      orc_destroy(o);
      return DML_E_ARG;
    }
    std::string line;
    std::getline(f, line);
    int nchunk = std::stoi(first_token(line));
    std::getline(f, line);
    for (int j = 0; j < nchunk; ++j) {
      std::getline(f, line);
      std::istringstream is(line);
      std::string sym;
      double x, y, zz;
      is >> sym >> x >> y >> zz;
      int h = s.new_atom();
      Atom& a = s.at[h];
      a.pos[0] = x;
      a.pos[1] = y;
      a.pos[2] = zz;
      s.setz(a, (sym == "CG" || sym == "cg") ? DML_Z_CG : DML_Z_LI);
      for (int k = 0; k < 3; ++k) {
        a.force[k] = 0.0;
        a.pos_old[k] = a.pos[k];
      }
      a.pos[2] = a.pos[2] + s.zmax;
      a.pos_old[2] = a.pos[2] + s.zmax;
      a.pbc[0] = a.pbc[1] = true;
      a.pbc[2] = false;
      s.chunk_list.push_back(h);
    }
  }
  s.try_ = 0;
  s.depo = 0;
  Frame last = s.frame();
  for (int i = 1; i <= c.nst; ++i) {
    s.step_body();
    if (s.err) break;
    if (i % c.nwr == 0) last = s.frame();
    s.step_tail();
  }
  int err = s.err;
  int n = (int)last.z.size();
  *n_out = n;
  if (zmax_out) *zmax_out = last.zmax;
  if (counters_out) {
    counters_out[0] = s.nupd;
    counters_out[1] = s.choques;
    counters_out[2] = s.choques2;
    counters_out[3] = s.choques3;
  }
  if (!err && n <= max_n) {
    std::memcpy(pos_out, last.pos.data(), sizeof(double) * 3 * n);
    for (int i = 0; i < n; ++i) z_out[i] = last.z[i];
  } else if (!err) {
    err = DML_E_ARG;
  }
  orc_destroy(o);
  return err;
}

}  // extern "C"

// Host build of the shared random-stream header, exported for tests that
// check it against libm and against the device build.
extern "C" {
void orc_rng_draw(uint64_t seed, int64_t step, uint64_t id, uint32_t stream, uint32_t sub,
                  uint32_t* out4) {
  dml_u4 w = dml_draw(seed, step, id, stream, sub);
  for (int k = 0; k < 4; ++k) out4[k] = w.w[k];
}
float orc_rng_logf(float x) { return dml_logf(x); }
void orc_rng_normal_pairs(const uint32_t* w, int64_t n_pairs, float* out) {
  for (int64_t i = 0; i < n_pairs; ++i)
    dml_normal_pair32f(w[2 * i], w[2 * i + 1], &out[2 * i], &out[2 * i + 1]);
}
void orc_rng_sincosf_2pi(float u, float* s, float* c) { dml_sincosf_2pi(u, s, c); }
void orc_rng_normal_quad(const uint32_t* w4, double* n4) {
  dml_u4 w;
  for (int k = 0; k < 4; ++k) w.w[k] = w4[k];
  dml_normal_quad(w, n4);
}
}
