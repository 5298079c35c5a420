// dml_api.cu - the C ABI of include/dml.h: context, device memory, the
// host-side constants of the reference (computed in its evaluation order),
// and the step sequence of src/dana.F90:173-265 queued on one stream and
// replayed as a CUDA graph.
//
// Host floating-point code in this file is compiled with
// -ffp-contract=off: the Ermak constants (set_ermak) and pair-table
// products are evaluated exactly as the reference evaluates them.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include <atomic>
#include <thread>

#include "../../include/dml.h"
#include "dml_internal.h"

using namespace dml;

constexpr int kScanMappings = 6;  // lanes per list row tried by the force-scan autotuner
constexpr double kThreadRowCand = 64.0;  // list build: one thread per row below this
constexpr int kCellFactors = 6;  // cell edge bounds tried by dml_tune_cells: 1.0, 1.1, .. 1.5

struct dml_ctx {
  dml_params P;
  KParams K;
  Dev D;
  cudaStream_t stream = nullptr;
  cudaStream_t aux = nullptr;  // captures conditional bodies
  int device = 0;
  bool loaded = false, setup_done = false;
  std::vector<dml_replica> reps;  // per-replica geometry and seeds
  std::vector<RepConst> rc;       // per-replica device constants (host copy)
  cudaGraphExec_t step_graph = nullptr;
  cudaGraphExec_t multi_graph = nullptr;  // graph_steps steps in one graph
  // chunk reservoir template (dml_set_chunk): positions as chunk.xyz gives
  // them, elements, chunk height
  std::vector<double> chunk_pos;
  std::vector<int> chunk_z;
  double chunk_dist = 0.0;
  int graph_steps = 100;
  bool scan_stale = true;  // the host changed the state: the next force scan is full
  int forced_lanes = 0;    // dml_set_scan_lanes (0: tuned)
  bool programmatic = true;  // kernel-to-kernel graph edges programmatic (programmatic_edges)
  int launches_per_step = 0;    // kernels of a step without a list rebuild
  int launches_per_rebuild = 0; // extra kernels when the list is rebuilt
  float tune_us[kScanMappings] = {};  // force-scan time per mapping (1, 2, 4, 8, 16, 32 lanes per row)
  double cell_factor = 1.0;           // chosen form: cell edge bound / (rc + skin)
  float cell_us[kCellFactors] = {};   // dml_tune_cells: time per step of each factor
  void* flush_buf = nullptr;
  std::string last_error;
  void* h_stage = nullptr;   // pinned staging of atom downloads, grown on demand
  size_t h_stage_bytes = 0;
  void* d_stage = nullptr;   // device packing of batch downloads, grown on demand
  size_t d_stage_bytes = 0;
  dml_observables* d_obs = nullptr;  // dml_salida's records, one per replica
  Scalars* h_sc = nullptr;  // pinned mirror of the per-replica state
  Global* h_g = nullptr;    // pinned mirror of the context-wide state
  std::vector<void*> allocs;
};

namespace {

int cuda_fail(dml_ctx* c, cudaError_t e, const char* what) {
  c->last_error = std::string(what) + ": " + cudaGetErrorString(e);
  return DML_E_CUDA;
}

#define CK(call)                                              \
  do {                                                        \
    cudaError_t _e = (call);                                  \
    if (_e != cudaSuccess) return cuda_fail(c, _e, #call);    \
  } while (0)

template <class T>
int dalloc(dml_ctx* c, T** p, size_t n) {
  size_t bytes = sizeof(T) * (n > 0 ? n : 1);
  cudaError_t e = cudaMalloc((void**)p, bytes);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaMalloc");
  c->allocs.push_back(*p);
  e = cudaMemsetAsync(*p, 0, bytes, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaMemset");
  return 0;
}

double pow6h(double x) {
  double x2 = x * x;
  double x4 = x2 * x2;
  return x2 * x4;
}

// Per-replica constants: box, cells (cgroup_tessellate, Cells.F90:227-242:
// ncells = int(box/(rc+skin)), cells off when all three are below 4).
// `edge`: the cell edge bound in units of rc + skin (1 as the reference;
// the chosen form's cell tuning takes larger cells, see dml_set_cell_factor).
void make_repconst(const dml_params& P, const dml_replica& r, RepConst& R, double edge = 1.0) {
  std::memset(&R, 0, sizeof R);
  for (int k = 0; k < 3; ++k) {
    R.box[k] = r.box[k];
    R.one_box[k] = 1.0 / r.box[k];
    R.halfbox[k] = r.box[k] * .5;
    R.boxf[k] = (float)r.box[k];
    R.halfboxf[k] = (float)(r.box[k] * .5);
  }
  double rcut_b = P.rc + P.skin;
  for (int k = 0; k < 3; ++k) R.ncells[k] = (int)(r.box[k] / rcut_b);
  R.use_cells = !(R.ncells[0] < 4 && R.ncells[1] < 4 && R.ncells[2] < 4);
  if (edge > 1.0 && R.use_cells)
    for (int k = 0; k < 3; ++k) {
      // larger cells, but never fewer than 3 along an axis that had 3 (no
      // stencil duplicates that the reference grid lacks)
      const int n = (int)(r.box[k] / (rcut_b * edge));
      R.ncells[k] = std::max(std::min(3, R.ncells[k]), n);
    }
  for (int k = 0; k < 3; ++k) {
    if (R.ncells[k] < 1) R.ncells[k] = 1;
    R.cell[k] = r.box[k] / (double)R.ncells[k];
    R.inv_cellf[k] = (float)(1.0 / R.cell[k]);
    R.cellf[k] = (float)R.cell[k];
    R.head_dim[k] = R.ncells[k] + 2;
  }
  R.ncell = R.use_cells ? R.head_dim[0] * R.head_dim[1] * R.head_dim[2] : 0;
  R.tess_hif = (float)((R.ncells[2] + 1) * R.cell[2]);
  R.seed = r.seed;
  // FP32 coordinates carry at most 2^-24 relative rounding; a difference of
  // two of them and its square stay well inside 64 ulps of maxc.
  const double maxc = 2.0 * std::max({r.box[0], r.box[1], r.box[2], r.zmax}) + 100.0;
  const double margin = std::max(1e-3, 64.0 * std::ldexp(maxc, -24));
  const double rl = P.rc + P.skin;
  R.margin = (float)margin;
  R.rlist_lo2 = (float)((rl - margin) * (rl - margin));
  R.rlist_hi2 = (float)((rl + margin) * (rl + margin));
  R.rc_lo2 = (float)((P.rc - margin) * (P.rc - margin));
  R.rc_hi2 = (float)((P.rc + margin) * (P.rc + margin));
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      R.r0f_pref2[i][j] = (float)((P.r0[i][j] + margin) * (P.r0[i][j] + margin));
  // gcmc_run's trial points lie in [z0, zmax]: their 27-cell stencils reach
  // the layers of those points and one more on either side, wrapped along z
  // like every stencil (Cells.F90:378-404); its cell sort covers only those.
  R.gl_all = 1;
  R.gl_mask = 0;
  const int nz = R.ncells[2];
  if (R.use_cells && P.reservoir == DML_RESERVOIR_GCMC && nz <= 62) {
    const int lo = std::max(0, (int)(r.z0 / R.cell[2]) + 1);
    const int hi = std::min(nz + 1, (int)(r.zmax / R.cell[2]) + 1);
    unsigned long long m = 0;
    for (int c = lo; c <= hi; ++c)
      for (int o = -1; o <= 1; ++o) m |= 1ull << (((c - 1 + o) % nz + 2 * nz) % nz + 1);
    if (lo <= hi && __builtin_popcountll(m) < nz) {
      R.gl_all = 0;
      R.gl_mask = m;
      // z is not periodic: a layer wrapped into a stencil from the far end of
      // the box lies farther than rc + skin in z from every trial point, so
      // none of its atoms can be a blocker or a list atom.  Its cells are
      // scanned (and read) empty; only the layers within reach are counted.
      const double reach = P.rc + P.skin + 1.0;
      unsigned long long cm = 0;
      for (int L = 1; L <= nz; ++L)
        if (((m >> L) & 1ull) && (double)L * R.cell[2] >= r.z0 - reach &&
            (double)(L - 1) * R.cell[2] <= r.zmax + reach)
          cm |= 1ull << L;
      R.gl_cmask = cm;
    }
  }
}

// Context-wide constants (see KParams).
void make_kparams(const dml_params& P, KParams& K) {
  std::memset(&K, 0, sizeof K);
  K.rc2 = P.rc * P.rc;
  double rl = P.rc + P.skin;
  K.rlist2 = rl * rl;
  K.skin = P.skin;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double r0 = P.r0[i][j], eps = P.eps[i][j];
      K.eps[i][j] = eps;
      K.r0sq[i][j] = r0 * r0;
      K.b0[i][j] = pow6h(r0);
      K.c0[i][j] = eps * 12.0 * K.b0[i][j];
      K.pair_on[i][j] = eps != 0.0;
      K.c12[i][j] = r0 > 0.0 ? 12.0 * eps / (r0 * r0) : 0.0;
    }
  for (int t = 0; t < 3; ++t) K.mass[t] = P.mass[t];
  for (int t = 0; t < 3; ++t) K.inv_mass[t] = 1.0 / P.mass[t];
  // set_ermak (dana.F90:947-971)
  const double h = P.h, gama = P.gamma;
  double cc0 = std::exp(-h * gama);
  double cc1 = (1.0 - cc0) / gama;
  double cc2 = (1.0 - cc1 / h) / gama;
  double sdr = std::sqrt(h / gama * (2.0 - (3.0 - 4.0 * cc0 + cc0 * cc0) / (h * gama)));
  double sdv = std::sqrt(1.0 - cc0 * cc0);
  double crv1 = (1.0 - cc0) * (1.0 - cc0) / (gama * sdr * sdv);
  double crv2 = std::sqrt(1.0 - (crv1 * crv1));
  double skt = std::sqrt(P.kb_driver * P.temp);
  K.cc0 = cc0;
  K.cc1 = cc1;
  K.cc2 = cc2;
  K.cc2h = cc2 * h;
  K.cc1mcc2 = cc1 - cc2;
  K.crv1 = crv1;
  K.crv2 = crv2;
  for (int t = 0; t < 3; ++t) {
    K.rfac[t] = skt / std::sqrt(P.mass[t]) * sdr;
    K.vfac[t] = skt / std::sqrt(P.mass[t]) * sdv;
  }
  // cbrownian_hs (dana.F90:817-823)
  K.fac_sc = std::sqrt(2.0 * P.dif_sc * P.h);
  K.fac_sei = std::sqrt(2.0 * P.dif_sei * P.h);
  K.dif_switch_z = P.dif_switch_z;
  K.h = P.h;
  K.prob = P.prob;
  K.h_over_tau = P.h / P.tau;
  K.ztop_is_z1 = P.reservoir == DML_RESERVOIR_CHUNKS ? 1.0 : 0.0;
  // piston: the step's second pbc_dispmax takes calc_rho's slab count
  K.rho_fused = P.reservoir == DML_RESERVOIR_PISTON;
  K.rcut_b = P.rc + P.skin;
  K.rhomedia = 5.775329e-4;  // dana.F90:445
  K.chunk_dist = 0.0;
  K.n_chunk = 0;
  K.integrator = P.integrator;
  K.reservoir = P.reservoir;
  K.mnb = P.mnb;
  K.ev_cap = P.event_cap;
  K.max_passes = P.max_passes;
  K.mixed = P.precision == DML_PRECISION_MIXED;
  K.scan_lanes = 16;  // until the step graph is tuned
  K.short_scan = 0;   // set with the tuned mapping (one lane per row)
  K.short_skin = 0.5f;
  K.near_lanes = 32;
  K.rcf = (float)P.rc;
  // 2^32 per eV/Å; 1 eV = 96.485 * 100 ui (dana.F90:23)
  K.fix_scale = std::ldexp(1.0, 32) / (96.485 * 100.0);
  K.fix_inv = 1.0 / K.fix_scale;
  K.act = P.act;
  K.beta_num = P.kb_module * P.temp;
  for (int t = 0; t < 3; ++t) K.beta_t[t] = std::sqrt(K.beta_num / P.mass[t]);
  K.nadj = P.nadj;
  K.cc0f = (float)K.cc0;
  K.cc1f = (float)K.cc1;
  K.cc2f = (float)K.cc2;
  K.cc2hf = (float)K.cc2h;
  K.cc1mcc2f = (float)K.cc1mcc2;
  K.crv1f = (float)K.crv1;
  K.crv2f = (float)K.crv2;
  for (int t = 0; t < 3; ++t) {
    K.rfacf[t] = (float)K.rfac[t];
    K.vfacf[t] = (float)K.vfac[t];
    K.inv_massf[t] = (float)K.inv_mass[t];
  }
  K.fac_scf = (float)K.fac_sc;
  K.fac_seif = (float)K.fac_sei;
  K.inv_hf = (float)(1.0 / P.h);
}

int read_scalars(dml_ctx* c) {
  if (c->loaded) {
    CK(cudaMemcpyAsync(c->h_g, c->D.g, sizeof(Global), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(c->h_sc, c->D.sc, sizeof(Scalars) * c->D.nrep, cudaMemcpyDeviceToHost,
                       c->stream));
  }
  CK(cudaStreamSynchronize(c->stream));
  return 0;
}

int write_scalars(dml_ctx* c) {
  CK(cudaMemcpyAsync(c->D.sc, c->h_sc, sizeof(Scalars) * c->D.nrep, cudaMemcpyHostToDevice,
                     c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return 0;
}

int finish(dml_ctx* c) {
  c->scan_stale = true;  // whatever the call did, the next step's force scan is full
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(c, e, "kernel launch");
  int rc = read_scalars(c);
  if (rc) return rc;
  if (c->h_g->error) {
    char buf[128];
    std::snprintf(buf, sizeof buf, "device error %d (%s), info %d", c->h_g->error,
                  dml_strerror(c->h_g->error), c->h_g->err_info);
    c->last_error = buf;
    return c->h_g->error;
  }
  return 0;
}

int set_step(dml_ctx* c, int64_t step) {
  long long v = step;
  CK(cudaMemcpyAsync(&c->D.g->step, &v, sizeof v, cudaMemcpyHostToDevice, c->stream));
  return 0;
}

// The kernel-to-kernel edges of a captured graph (a conditional body is a
// graph of its own and is passed here separately) made programmatic at the
// kernel-exit port: a kernel is launched once every block of the kernel it
// follows has exited (none of our kernels triggers earlier), and waits at its
// first statement (DML_GRID_WAIT) until that kernel's writes are visible.
// This saves part of the launch gap: 1.170 -> 1.163 ms on the config-5 step
// graph, 2.003 -> 1.992 ms on config 4.  The launch-completion port (blocks
// resident as soon as every block of the predecessor has started) made the
// config-5 step slower, 1.180 -> 1.306 ms.  Edges from or to other nodes
// (copies, memsets, conditional nodes) keep full serialisation.  If the
// runtime refuses the programmatic edges, the default ones are put back.
cudaError_t programmatic_edges(cudaGraph_t g) {
  size_t n = 0;
  cudaError_t e = cudaGraphGetEdges(g, nullptr, nullptr, nullptr, &n);
  if (e != cudaSuccess || n == 0) return e;
  std::vector<cudaGraphNode_t> from(n), to(n);
  std::vector<cudaGraphEdgeData> ed(n);
  e = cudaGraphGetEdges(g, from.data(), to.data(), ed.data(), &n);
  if (e != cudaSuccess) return e;
  std::vector<cudaGraphNode_t> kf, kt;
  for (size_t i = 0; i < n; ++i) {
    if (ed[i].type != cudaGraphDependencyTypeDefault || ed[i].from_port != 0 || ed[i].to_port != 0)
      continue;
    cudaGraphNodeType a, b;
    if (cudaGraphNodeGetType(from[i], &a) != cudaSuccess ||
        cudaGraphNodeGetType(to[i], &b) != cudaSuccess)
      continue;
    if (a == cudaGraphNodeTypeKernel && b == cudaGraphNodeTypeKernel) {
      kf.push_back(from[i]);
      kt.push_back(to[i]);
    }
  }
  if (kf.empty()) return cudaSuccess;
  e = cudaGraphRemoveDependencies(g, kf.data(), kt.data(), nullptr, kf.size());
  if (e != cudaSuccess) return e;
  std::vector<cudaGraphEdgeData> pe(kf.size());
  for (auto& x : pe) {
    std::memset(&x, 0, sizeof x);
    x.from_port = cudaGraphKernelNodePortProgrammatic;
    x.type = cudaGraphDependencyTypeProgrammatic;
  }
  e = cudaGraphAddDependencies(g, kf.data(), kt.data(), pe.data(), kf.size());
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    return cudaGraphAddDependencies(g, kf.data(), kt.data(), nullptr, kf.size());
  }
  return cudaSuccess;
}

// test_update inside a graph capture: the displacement-test kernel sets the
// condition of an IF node whose body is the rebuild (update(), Neighbor.F90:
// 608-633), so steps without a rebuild launch no rebuild kernel at all.
int capture_test_update(dml_ctx* c, int* n_base, int* n_body, bool near_in_body, bool second) {
  cudaStream_t s = c->stream;
  cudaStreamCaptureStatus st;
  cudaGraph_t g;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  CK(cudaStreamGetCaptureInfo(s, &st, nullptr, &g, &deps, nullptr, &nd));
  cudaGraphConditionalHandle h;
  CK(cudaGraphConditionalHandleCreate(&h, g, 0, 0));
  *n_base += k_pbc_dispmax_cond(c->D, c->K, c->D.cap, h, s, second);
  CK(cudaStreamGetCaptureInfo(s, &st, nullptr, &g, &deps, nullptr, &nd));
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h;
  cp.conditional.type = cudaGraphCondTypeIf;
  cp.conditional.size = 1;
  cudaGraphNode_t node;
  CK(cudaGraphAddNode(&node, g, deps, nullptr, nd, &cp));
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  CK(cudaStreamBeginCaptureToGraph(c->aux, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
  *n_body += k_rebuild(c->D, c->K, c->D.cap, c->D.cap, c->D.cap, c->aux);
  // the rebuilt lists need overlap_moveback's near entries searched again
  if (near_in_body) *n_body += k_overlap_detect(c->D, c->K, c->D.cap, 2, c->aux);
  cudaGraph_t outg;
  CK(cudaStreamEndCapture(c->aux, &outg));
  if (c->programmatic) CK(programmatic_edges(outg));
  CK(cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  return 0;
}

// bloques (dana.F90:247, 716-773) and the test_update it ends with: the
// chunk kernel, then the rebuild of the replicas that took a chunk -- a
// conditional graph node under capture, else decided on the host.  The
// displacement test runs for every replica; those without a chunk decide
// what their second test_update of the step decided (nothing has moved since).
int queue_bloques(dml_ctx* c, bool capture, int* n_base, int* n_body) {
  cudaStream_t s = c->stream;
  *n_base += k_bloques(c->D, c->K, s);
  if (capture) {
    cudaStreamCaptureStatus st;
    cudaGraph_t g;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    CK(cudaStreamGetCaptureInfo(s, &st, nullptr, &g, &deps, nullptr, &nd));
    cudaGraphConditionalHandle h;
    CK(cudaGraphConditionalHandleCreate(&h, g, 0, 0));
    *n_base += k_chunk_cond(c->D, h, s);
    CK(cudaStreamGetCaptureInfo(s, &st, nullptr, &g, &deps, nullptr, &nd));
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeIf;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    CK(cudaGraphAddNode(&node, g, deps, nullptr, nd, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    CK(cudaStreamBeginCaptureToGraph(c->aux, body, nullptr, nullptr, 0,
                                     cudaStreamCaptureModeRelaxed));
    *n_body += k_rank_prefix(c->D, c->aux);
    *n_body += k_test_update(c->D, c->K, c->D.cap, c->D.cap, c->D.cap, c->aux);
    cudaGraph_t outg;
    CK(cudaStreamEndCapture(c->aux, &outg));
    if (c->programmatic) CK(programmatic_edges(outg));
    CK(cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1,
                                           cudaStreamSetCaptureDependencies));
    return 0;
  }
  int ev = 0;
  CK(cudaMemcpyAsync(&ev, &c->D.g->chunk_event, sizeof ev, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (ev) {
    *n_body += k_rank_prefix(c->D, s);
    *n_body += k_test_update(c->D, c->K, c->D.cap, c->D.cap, c->D.cap, s);
  }
  return 0;
}

// One iteration of the loop body of dana.F90:173-265 (without salida,
// timer_dump and the chunk reservoir), queued on the context stream.  With
// `ev` (DML_NPHASE + 1 events) the phase boundaries are recorded.  With
// `capture` the rebuilds become conditional graph nodes.  Returns 0 or a
// status; the kernels queued are counted in *n_base (every step) and *n_body
// (only when the list is rebuilt).
// An idle stretch of the stream inside a profiled phase (a host read of the
// rebuild condition), subtracted from that phase's time.
struct ProfileGap {
  cudaEvent_t a, b;
  int phase;
};

int enqueue_step(dml_ctx* c, cudaEvent_t* ev, bool capture, int* n_base, int* n_body,
                 std::vector<ProfileGap>* gaps = nullptr) {
  const Dev& d = c->D;
  const KParams& k = c->K;
  cudaStream_t s = c->stream;
  const int cap = d.cap;  // kernels read the live counts from the device scalars
  int n = 0, nb = 0, rc = 0;
  auto mark = [&](int i) {
    if (ev) cudaEventRecord(ev[i], s);
  };
  const bool ermak_ = c->P.integrator == DML_INTEGRATOR_ERMAK;
  auto test_update = [&](bool first) -> int {
    if (capture) return capture_test_update(c, &n, &nb, first && ermak_, !first);
    if (gaps) {
      // the graph's kernels: the rebuild (and the near search after the
      // first one) only when some replica rebuilds, decided on the host
      n += k_pbc_dispmax(d, k, cap, s, !first);
      ProfileGap gp;
      gp.phase = first ? DML_PHASE_TEST_UPDATE1 : DML_PHASE_TEST_UPDATE2;
      CK(cudaEventCreate(&gp.a));
      CK(cudaEventCreate(&gp.b));
      CK(cudaEventRecord(gp.a, s));
      int any = 0;
      CK(cudaMemcpyAsync(&any, &d.g->any_rebuild, sizeof any, cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      CK(cudaEventRecord(gp.b, s));
      gaps->push_back(gp);
      if (any) {
        nb += k_rebuild(d, k, cap, cap, cap, s);
        if (first && ermak_) nb += k_overlap_detect(d, k, cap, 2, s);
      }
      return 0;
    }
    n += k_test_update(d, k, cap, cap, cap, s, !first);
    return 0;
  };
  mark(DML_PHASE_INTEGRATE);
  const bool ermak = c->P.integrator == DML_INTEGRATOR_ERMAK;
  n += k_step_begin(d, ermak ? 0 : 1, s);
  n += k_rank_prefix(d, s);
  if (ermak) {
    n += k_ermak_a(d, k, cap, s);  // + overlap_moveback's reset and delta
    mark(DML_PHASE_FORCE_PAIRS);
    n += k_force_pairs(d, k, cap, true, s);  // + overlap_moveback's near entries
    mark(DML_PHASE_FORCE_SUM);
    n += k_force_sum(d, k, cap, true, s);  // fuerza + ermak_b
  } else {
    n += k_brownian(d, k, cap, s);  // + overlap_moveback's reset and delta
    mark(DML_PHASE_FORCE_PAIRS);
    mark(DML_PHASE_FORCE_SUM);
  }
  mark(DML_PHASE_TEST_UPDATE1);
  if ((rc = test_update(true)) != 0) return rc;
  mark(DML_PHASE_OVERLAP);
  // near entries: found by the force scan (Ermak), searched again inside
  // the first test_update's rebuild node (graph) or when stale (eager);
  // the Brownian step has no force scan and always searches here
  n += k_overlap(d, k, cap, cap, false, !ermak ? 2 : (capture || gaps ? 0 : 1), s);
  mark(DML_PHASE_TEST_UPDATE2);
  if ((rc = test_update(false)) != 0) return rc;
  mark(DML_PHASE_COMMIT);
  n += k_capture_commit(d, k, cap, s);
  mark(DML_PHASE_GCMC_CELLS);
  if (c->P.reservoir == DML_RESERVOIR_GCMC) n += k_gcmc_cells(d, k, cap, s);
  mark(DML_PHASE_GCMC);
  if (c->P.reservoir == DML_RESERVOIR_GCMC) n += k_gcmc_trials(d, k, s);
  mark(DML_PHASE_RHO_PISTON);
  if (!k.rho_fused) n += k_calc_rho(d, k, cap, s);  // else taken by the second test_update
  if (c->P.reservoir == DML_RESERVOIR_PISTON) n += k_piston(d, k, cap, s);
  if (c->P.reservoir == DML_RESERVOIR_CHUNKS && (rc = queue_bloques(c, capture, &n, &nb)) != 0)
    return rc;
  mark(DML_NPHASE);
  if (n_base) *n_base = n;
  if (n_body) *n_body = nb;
  return 0;
}

// Autotuner of the thread mapping of the step's per-row scan: the force
// scan (Ermak) or the near-contact search of overlap_moveback (Brownian,
// which has no force scan and searches every step).  Each mapping (1, 2, 4,
// 8, 16 or 32 lanes per list row) scans the loaded lists a few times and the
// fastest is kept for the step graph.  The trial scans change nothing the
// next step reads: the candidate queue is cleared after each one, and the
// near entries, unions and active flags are reset or rewritten by every
// step before they are used.  Row lengths depend on the skin, the density
// and the electrode, so the best mapping is a property of the workload.
int autotune_scan(dml_ctx* c) {
  cudaStream_t s = c->stream;
  const bool ermak = c->P.integrator == DML_INTEGRATOR_ERMAK;
  const int lanes[kScanMappings] = {1, 2, 4, 8, 16, 32};
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  k_rank_prefix(c->D, s);
  KParams k = c->K;
  // near: the near-contact search of overlap_moveback (every step with the
  // Brownian integrator; with Ermak only over the rows of replicas whose
  // list was just rebuilt, the force scan finding the near entries
  // otherwise), else the force scan.
  auto scan = [&](bool near) {
    if (!near) {
      k_force_scan(c->D, k, c->D.cap, false, s);
      k_reset_candidates(c->D, s);
    } else {
      k_overlap_detect(c->D, k, c->D.cap, 0, s);
    }
  };
  // Mappings in order of lanes; the search stops at the first one that is
  // slower than the previous and than 1.25x the best (times grow with the
  // lanes past the best); untimed mappings keep tune_us 0.
  auto sweep = [&](bool near, float* us) -> int {
    float best = 1e30f, prev = 1e30f;
    int best_l = 32;
    for (int v = 0; v < kScanMappings; ++v) {
      k.scan_lanes = lanes[v];
      k.near_lanes = lanes[v];
      scan(near);  // warm-up
      float ms = 0;
      if (cudaEventRecord(e0, s) != cudaSuccess) return -1;
      for (int rep = 0; rep < 3; ++rep) scan(near);
      if (cudaEventRecord(e1, s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
          cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
        return -1;
      if (us) us[v] = ms * 1e3f / 3.0f;
      if (ms < best) {
        best = ms;
        best_l = lanes[v];
      }
      if (ms > prev && ms > 1.25f * best) break;
      prev = ms;
    }
    return best_l;
  };
  int sl = 0, nl = 0;
  if (ermak) {
    sl = c->forced_lanes > 0 ? c->forced_lanes : sweep(false, c->tune_us);
    nl = sl < 0 ? -1 : sweep(true, nullptr);
  } else {
    nl = c->forced_lanes > 0 ? c->forced_lanes : sweep(true, c->tune_us);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (sl < 0 || nl < 0) return cuda_fail(c, cudaGetLastError(), "autotune timing");
  if (ermak) c->K.scan_lanes = sl;
  c->K.near_lanes = nl;
  // The force scan walks only flagged rows between full scans when a step
  // moves atoms by their integrator alone (no piston, no chunk shifts) and
  // the scan runs one lane per row.
  c->K.short_scan = ermak && sl == 1 && c->P.reservoir != DML_RESERVOIR_PISTON &&
                    c->P.reservoir != DML_RESERVOIR_CHUNKS;
  return finish(c);
}

int build_step_graph(dml_ctx* c) {
  if (c->step_graph) return 0;
  int trc = autotune_scan(c);
  if (trc) return trc;
  cudaGraph_t g;
  CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed));
  int nb = 0, nr = 0;
  int rc = enqueue_step(c, nullptr, true, &nb, &nr);
  cudaError_t e = cudaStreamEndCapture(c->stream, &g);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamEndCapture");
  if (c->programmatic) e = programmatic_edges(g);
  if (e == cudaSuccess) e = cudaGraphInstantiate(&c->step_graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaGraphInstantiate");
  c->launches_per_step = nb;
  c->launches_per_rebuild = nr / 2;
  return 0;
}

// graph_steps iterations of the loop body captured into one graph (each
// with its own conditional rebuild nodes), so that a run of many steps is a
// few graph launches.
int build_multi_graph(dml_ctx* c) {
  if (c->multi_graph) return 0;
  int rc = build_step_graph(c);
  if (rc) return rc;
  cudaGraph_t g;
  CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed));
  for (int i = 0; i < c->graph_steps && rc == 0; ++i) {
    int nb = 0, nr = 0;
    rc = enqueue_step(c, nullptr, true, &nb, &nr);
  }
  cudaError_t e = cudaStreamEndCapture(c->stream, &g);
  if (rc) {
    if (e == cudaSuccess) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamEndCapture (multi-step graph)");
  if (c->programmatic) e = programmatic_edges(g);
  if (e == cudaSuccess) e = cudaGraphInstantiate(&c->multi_graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaGraphInstantiate (multi-step graph)");
  return 0;
}

// nsteps iterations: as many graph_steps-step graphs as fit, then one-step
// graphs.
// Before steps queued after any other call: every replica's next force scan
// is full (the flags of the partial scans belong to the state the steps left).
void scan_refresh(dml_ctx* c) {
  if (!c->scan_stale) return;
  k_scan_invalidate(c->D, c->stream);
  c->scan_stale = false;
}

int queue_steps(dml_ctx* c, int64_t nsteps) {
  int rc = build_step_graph(c);
  if (rc) return rc;
  scan_refresh(c);
  int64_t i = 0;
  if (c->graph_steps > 1 && nsteps >= c->graph_steps) {
    if ((rc = build_multi_graph(c)) != 0) return rc;
    for (; i + c->graph_steps <= nsteps; i += c->graph_steps)
      CK(cudaGraphLaunch(c->multi_graph, c->stream));
  }
  for (; i < nsteps; ++i) CK(cudaGraphLaunch(c->step_graph, c->stream));
  return 0;
}

constexpr size_t kFlushBytes = 256ull << 20;  // > 2x the 129 MB L2

int ensure_flush(dml_ctx* c) {
  if (c->flush_buf) return 0;
  CK(cudaMalloc(&c->flush_buf, kFlushBytes));
  return 0;
}

}  // namespace

extern "C" {

void dml_params_default(dml_params* p) {
  std::memset(p, 0, sizeof *p);
  // program dana (dana.F90:22-24): kB_ui = kB_eVK * eV_ui, eV_ui = 96.485 * 100.
  const double eV_ui = 96.485 * 100.0;
  // gems_constants (Constants.F90:105-167): kB_ui = kB_ev / (axps_mxs^2 uma_kg joule_ev).
  const double joule_ev = 1.0 / 1.60219e-19;
  const double ui_ev = 1.0e2 * 1.0e2 * 1.6605402e-27 * joule_ev;
  const double ev_ui = 1.0 / ui_ev;
  p->box[0] = 100.0;
  p->box[1] = 100.0;
  p->box[2] = 200.0;
  p->z0 = 100.0;
  p->zmax = 200.0;
  p->h = 1.e-2;
  p->gamma = 1.0;
  p->temp = 300.0;
  p->kb_driver = 8.617330350e-5 * eV_ui;
  p->kb_module = 8.617385e-05 * ev_ui;
  // Pair tables (dana.F90:86-100), index [z-1][z-1]: 1 Li, 2 CG, 3 F.
  p->r0[1][0] = p->r0[0][1] = 3.5;
  p->eps[0][0] = 2313.6;
  p->r0[0][0] = 3.2;
  p->eps[2][2] = 121.0;
  p->r0[2][2] = 3.61;
  p->eps[0][2] = p->eps[2][0] = 529.1;
  p->r0[0][2] = p->r0[2][0] = 1.564;
  p->mass[0] = p->mass[1] = p->mass[2] = 6.94;
  p->rc = 3.2;
  p->skin = 10.0;
  p->prob = 1.0;
  p->dif_sc = 250.0;
  p->dif_sei = 250.0;
  p->dif_switch_z = 80.0;
  p->tau = 0.1;
  p->integrator = DML_INTEGRATOR_ERMAK;
  p->reservoir = DML_RESERVOIR_PISTON;
  p->precision = DML_PRECISION_FP64;
  p->mnb = 1024;
  p->max_passes = 64;
  p->event_cap = 64;
}

const char* dml_strerror(int code) {
  switch (code) {
    case DML_OK: return "ok";
    case DML_E_ARG: return "invalid argument";
    case DML_E_CUDA: return "CUDA error";
    case DML_E_NOMEM: return "out of memory";
    case DML_E_OUT_OF_TESSELLATION: return "Particle out of tessellation";
    case DML_E_UNSORT: return "Unsort cgroup particle fail";
    case DML_E_INDEX: return "Index inconsistency";
    case DML_E_NO_PARTICLES: return "No more particles";
    case DML_E_CHOSEN_MISSING: return "Chosen particle does not exists";
    case DML_E_RESERVOIR: return "Unknown reservoir type";
    case DML_E_DENDRITE: return "deposit above z0 (dendrite reached the reservoir)";
    case DML_E_RSA: return "maximum number of placement tries reached";
    case DML_E_OVERLAP_PASSES: return "overlap_moveback exceeded the pass cap";
    case DML_E_NEIGH_OVERFLOW: return "more neighbours than mnb";
    case DML_E_EVENT_OVERFLOW: return "too many interacting entries for one atom";
    case DML_E_FIXEDPOINT_OVERFLOW: return "force beyond the fixed-point range";
    case DML_E_CAPACITY: return "atom capacity exceeded";
    case DML_E_UNSUPPORTED: return "option not supported on the device";
    case DML_E_NEAR_OVERFLOW: return "too many near contacts";
    case DML_E_STATE: return "call out of order";
    default: return "unknown error";
  }
}

const char* dml_last_error(dml_ctx* c) { return c ? c->last_error.c_str() : "no context"; }

int dml_create_batch(const dml_params* p, int32_t n_rep, const dml_replica* reps,
                     dml_ctx** out) {
  if (!p || !out || n_rep <= 0 || !reps) return DML_E_ARG;
  *out = nullptr;
  if (p->reservoir < 0 || p->reservoir > 3) return DML_E_RESERVOIR;
  if (p->reservoir == DML_RESERVOIR_GCMC && (p->nadj < 0 || !(p->act > 0))) return DML_E_ARG;
  if (p->precision != DML_PRECISION_FP64 && p->precision != DML_PRECISION_MIXED) return DML_E_ARG;
  if (!(p->h > 0 && p->rc > 0)) return DML_E_ARG;
  // The FP32 pre-filters assume the minimum image is unambiguous at every cut-off.
  double rmax = p->rc + p->skin;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) rmax = std::max(rmax, p->r0[i][j]);
  for (int r = 0; r < n_rep; ++r) {
    const dml_replica& q = reps[r];
    if (!(q.box[0] > 0 && q.box[1] > 0 && q.box[2] > 0)) return DML_E_ARG;
    if (q.box[0] * 0.5 <= rmax + 0.01 || q.box[1] * 0.5 <= rmax + 0.01) return DML_E_ARG;
  }
  dml_ctx* c = new dml_ctx();
  c->P = *p;
  if (c->P.mnb <= 0) c->P.mnb = 1024;
  if (c->P.max_passes <= 0) c->P.max_passes = 64;
  if (c->P.event_cap <= 0) c->P.event_cap = 64;
  if (c->P.event_cap > 128) c->P.event_cap = 128;
  c->reps.assign(reps, reps + n_rep);
  make_kparams(c->P, c->K);
  c->rc.resize(n_rep);
  for (int r = 0; r < n_rep; ++r) make_repconst(c->P, reps[r], c->rc[r]);
  cudaError_t e = cudaGetDevice(&c->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->aux, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMallocHost((void**)&c->h_sc, sizeof(Scalars) * n_rep);
  if (e == cudaSuccess) e = cudaMallocHost((void**)&c->h_g, sizeof(Global));
  if (e != cudaSuccess) {
    dml_destroy(c);
    return DML_E_CUDA;
  }
  std::memset(c->h_g, 0, sizeof(Global));
  std::memset(c->h_sc, 0, sizeof(Scalars) * n_rep);
  c->D.nrep = n_rep;
  *out = c;
  return 0;
}

int dml_create(const dml_params* p, dml_ctx** out) {
  if (!p) return DML_E_ARG;
  dml_replica r;
  std::memset(&r, 0, sizeof r);
  for (int k = 0; k < 3; ++k) r.box[k] = p->box[k];
  r.z0 = p->z0;
  r.zmax = p->zmax;
  r.z1 = p->z1;
  r.seed = p->seed;
  return dml_create_batch(p, 1, &r, out);
}

int dml_num_replicas(dml_ctx* c) { return c ? c->D.nrep : -DML_E_ARG; }

void dml_destroy(dml_ctx* c) {
  if (!c) return;
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->step_graph) cudaGraphExecDestroy(c->step_graph);
  if (c->multi_graph) cudaGraphExecDestroy(c->multi_graph);
  for (void* p : c->allocs) cudaFree(p);
  if (c->flush_buf) cudaFree(c->flush_buf);
  if (c->h_sc) cudaFreeHost(c->h_sc);
  if (c->h_stage) cudaFreeHost(c->h_stage);
  if (c->d_stage) cudaFree(c->d_stage);
  if (c->d_obs) cudaFree(c->d_obs);
  if (c->h_g) cudaFreeHost(c->h_g);
  if (c->stream) cudaStreamDestroy(c->stream);
  if (c->aux) cudaStreamDestroy(c->aux);
  delete c;
}

int dml_set_atoms_batch(dml_ctx* c, const dml_atoms* atoms) {
  if (!c || !atoms) return DML_E_ARG;
  if (c->loaded) return DML_E_STATE;
  // The runtime's last-error slot is shared by every caller in the process:
  // clear what an earlier call left there, so that the launch checks below
  // report this call's own launches.
  (void)cudaGetLastError();
  const int nrep = c->D.nrep;
  Dev& d = c->D;
  // capacities: positions per replica, a multiple of kSpan
  // positions are indexed with int on the device: a context holds at most
  // kMaxPositions of them (far beyond what HBM holds at this layout)
  constexpr long long kMaxPositions = 1LL << 30;
  int total = 0, ncell = 0, any_cells = 0, any_verlet = 0, n_cch = 0;
  const bool chunks = c->P.reservoir == DML_RESERVOIR_CHUNKS;
  const int n_chunk = (int)c->chunk_z.size();
  if (chunks && n_chunk == 0) {
    c->last_error = "chunk reservoir: dml_set_chunk must come before the atoms";
    return DML_E_STATE;
  }
  for (int r = 0; r < nrep; ++r) {
    const dml_atoms* a = atoms + r;
    if (a->n <= 0 || !a->pos || !a->z) return DML_E_ARG;
    // room for 16 chunks by default with the chunk reservoir
    const long long want = c->P.capacity > 0 ? c->P.capacity
                           : (c->P.reservoir == DML_RESERVOIR_GCMC ? 2LL * a->n + 1024
                              : chunks ? a->n + 16LL * n_chunk : a->n);
    const long long capl = (std::max<long long>(a->n, want) + kSpan - 1) / kSpan * kSpan;
    if (total + capl > kMaxPositions) {
      c->last_error = "capacity: more than 2^30 atom positions in one context";
      return DML_E_CAPACITY;
    }
    const int cap = (int)capl;
    RepConst& R = c->rc[r];
    // The chunk reservoir raises the box by the chunk height at each chunk,
    // at most (cap - n) / n_chunk times: the replica's cells (and its FP32
    // pre-filter margins) are sized for the tallest box.
    RepConst M = R;
    if (chunks) {
      dml_replica tall = c->reps[r];
      const long long events = (cap - a->n) / n_chunk;
      tall.zmax = c->reps[r].zmax + (double)events * c->chunk_dist;
      tall.box[2] = std::max(c->reps[r].box[2], tall.zmax);
      make_repconst(c->P, tall, M);
      R.margin = M.margin;
      R.rlist_lo2 = M.rlist_lo2;
      R.rlist_hi2 = M.rlist_hi2;
      R.rc_lo2 = M.rc_lo2;
      R.rc_hi2 = M.rc_hi2;
      std::memcpy(R.r0f_pref2, M.r0f_pref2, sizeof R.r0f_pref2);
    }
    R.base = total;
    R.cap = cap;
    R.nblk = cap / kSpan;
    R.cell_off = ncell;
    R.cch0 = n_cch;
    n_cch += (M.ncell + kCellChunk - 1) / kCellChunk;
    ncell += M.ncell + (M.use_cells ? 1 : 0);  // + the replica's sentinel cell
    total += cap;
    if (R.use_cells || M.use_cells) any_cells = 1;
    if (!R.use_cells) any_verlet = 1;
  }
  d.cap = total;
  d.max_rep_cap = 0;
  d.gcmc_rows = 0;
  for (int r = 0; r < nrep; ++r) {
    const RepConst& R = c->rc[r];
    d.max_rep_cap = std::max(d.max_rep_cap, R.cap);
    // rows of gcmc_run's shared-memory sort; larger replicas run sequentially
    if (R.use_cells) d.gcmc_rows = std::max(d.gcmc_rows, std::min(R.head_dim[1] * R.head_dim[2], 16384));
  }
  d.ncell_tot = ncell;
  d.n_cch = n_cch;
  d.any_cells = any_cells;
  d.any_verlet = any_verlet;
  // List build mapping per replica: one thread per row where the 27 cells
  // around an atom hold few candidates (below kThreadRowCand on average at
  // loading), a warp per row elsewhere.  Both give the same rows.
  d.any_list_thread = 0;
  d.any_list_warp = 0;
  for (int r = 0; r < nrep; ++r) {
    RepConst& R = c->rc[r];
    const double cells = (double)R.ncells[0] * R.ncells[1] * R.ncells[2];
    const double cand = 27.0 * atoms[r].n / cells;
    R.list_thread = cand <= kThreadRowCand ? 1 : 0;
    if (R.list_thread) d.any_list_thread = 1; else d.any_list_warp = 1;
  }
  const int cap = total;
  c->K.cand_cap = (int)std::min<long long>(16LL * cap, 1LL << 30);  // writes are bounded by it
  int rc = 0;
#define AL(ptr, cnt) \
  if ((rc = dalloc(c, &(ptr), (cnt))) != 0) return rc;
  AL(d.pos, cap);
  AL(d.vel, cap);
  AL(d.acel, cap);
  AL(d.force, cap);
  AL(d.old_cg, cap);
  AL(d.pos_old, cap);
  AL(d.ranv, c->P.precision == DML_PRECISION_MIXED ? 1 : (size_t)cap);
  AL(d.ranvf, c->P.precision == DML_PRECISION_MIXED ? (size_t)cap : 1);
  AL(d.posf, cap);
  AL(d.posf_old, cap);
  AL(d.epot, cap);
  AL(d.typ, cap);
  AL(d.skip, cap);
  AL(d.state, cap);
  AL(d.active, cap);
  AL(d.id, cap);
  AL(d.rank, cap);
  AL(d.bslot, cap);
  AL(d.ref, cap);
  AL(d.b2hs, cap);
  AL(d.nn, cap);
  AL(d.list, (size_t)cap * c->P.mnb);
  AL(d.cell_of, cap);
  AL(d.cell_count, ncell + 1);
  AL(d.cell_start, ncell + 1);
  AL(d.cell_fill, ncell + 1);
  AL(d.cell_atoms, cap);
  AL(d.alist, cap);
  AL(d.apos, cap);
  AL(d.gorder, cap);
  AL(d.gpos, cap);
  AL(d.in_gcmc, cap);
  AL(d.ins_head, ncell + 1);
  AL(d.ins_next, cap);
  // only the form in use gets its force accumulators
  const bool mixed = c->P.precision == DML_PRECISION_MIXED;
  AL(d.facc, mixed ? 4 * (size_t)cap : 4);
  AL(d.ftouch, mixed ? (size_t)cap / 32 + 1 : 1);
  AL(d.fnz, mixed ? (size_t)cap / 32 + 1 : 1);
  AL(d.ftlist, mixed ? (size_t)cap : 1);
  AL(d.flist, cap);
  AL(d.cand, (size_t)c->K.cand_cap);
  AL(d.ev_count, cap);
  AL(d.ev, mixed ? 1 : (size_t)cap * c->P.event_cap);
  AL(d.near_count, cap);
  AL(d.near, (size_t)cap * kNearCap);
  AL(d.uf, cap);
  AL(d.comp_size, cap);
  AL(d.comp_id, cap);
  AL(d.comp_rank, cap);
  AL(d.comp_fill, cap);
  AL(d.comp_members, cap);
  AL(d.comp_list, 2 * (size_t)cap);
  AL(d.act_list, cap);
  AL(d.act_big_pre, nrep + 1);
  AL(d.rowflag, cap);
  AL(d.sl_rows, cap);
  AL(d.sl_pre, nrep + 1);
  AL(d.sl_nrows, nrep);
  AL(d.glist, c->P.reservoir == DML_RESERVOIR_GCMC ? (size_t)cap : 1);
  AL(d.pr_cnt, (size_t)nrep * kCntStride);
  d.nblk_part = cap / kBlock + 1;
  AL(d.part, 2 * (size_t)d.nblk_part);
  AL(d.part1, 2 * (size_t)d.nblk_part);
  AL(d.xspan, (size_t)cap / kSpan + 1);
  AL(d.xpart, 2 * ((size_t)cap / kSpan + 1));
  AL(d.part_cnt, 2 * (size_t)d.nblk_part);
  AL(d.dirty, (size_t)d.nblk_part);
  AL(d.sc, nrep);
  AL(d.g, 1);
  AL(d.rc, nrep);
  AL(d.rep_of, cap);
  AL(d.rank_pre, nrep + 1);
  AL(d.reb_pre, nrep + 1);
  AL(d.rebc_pre, nrep + 1);
  AL(d.chunk_sum, n_cch > 0 ? n_cch : 1);
  AL(d.chunk_base, n_cch > 0 ? n_cch : 1);
  AL(d.big_cells, ncell + 1);
  AL(d.cch_rep, n_cch > 0 ? n_cch : 1);
  {
    // every chunk of the replicas' cell ranges (those sized for a taller box
    // included) belongs to its replica
    std::vector<int> cr(n_cch > 0 ? n_cch : 1, 0);
    for (int r = 0; r < nrep; ++r) {
      const int end = r + 1 < nrep ? c->rc[r + 1].cch0 : n_cch;
      for (int q = c->rc[r].cch0; q < end; ++q) cr[q] = r;
    }
    // on the context stream, after the zeroing of the new allocation
    CK(cudaMemcpyAsync(d.cch_rep, cr.data(), sizeof(int) * cr.size(), cudaMemcpyHostToDevice,
                       c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  AL(d.chk_pos, chunks ? (size_t)nrep * n_chunk : 1);
  AL(d.chk_pold, chunks ? (size_t)nrep * n_chunk : 1);
  AL(d.chk_typ, chunks ? (size_t)n_chunk : 1);
  if (c->P.reservoir == DML_RESERVOIR_GCMC) {
    const bool par = c->P.nadj <= kGcmcMaxTrials;
    AL(d.grp, nrep);
    AL(d.gpre, par ? (size_t)nrep * kGcmcMaxTrials : 1);
    AL(d.gpm, par ? (size_t)nrep * kGcmcMaxTrials * kGcmcMaskW : 1);
    AL(d.glp, par ? (size_t)cap : 1);
    AL(d.gsort, par ? (size_t)cap : 1);
    AL(d.gw_mem, par ? (size_t)cap / 32 : 1);
    AL(d.gw_slab, par ? (size_t)cap / 32 : 1);
  }
#undef AL

  // Compact upload: the caller's arrays concatenated over the replicas in one
  // host buffer, one copy, and load_atoms_kernel expanding them into the
  // position layout (replica r at [base, base + cap)).  Positions no atom
  // takes keep the zero fill of dalloc or the -1 fill below.
  std::vector<int> off(nrep + 1, 0);
  for (int r = 0; r < nrep; ++r) off[r + 1] = off[r] + atoms[r].n;
  const int n_tot = off[nrep];
  auto any_of = [&](auto field) {
    for (int r = 0; r < nrep; ++r)
      if (atoms[r].*field) return true;
    return false;
  };
  const bool has_vel = any_of(&dml_atoms::vel), has_acel = any_of(&dml_atoms::acel),
             has_force = any_of(&dml_atoms::force), has_pold = any_of(&dml_atoms::pos_old),
             has_ocg = any_of(&dml_atoms::old_cg), has_epot = any_of(&dml_atoms::epot),
             has_skip = any_of(&dml_atoms::skip), has_id = any_of(&dml_atoms::id);
  // section offsets in the staging buffer, each 16-byte aligned
  size_t nb = 0;
  auto sec = [&](bool on, size_t bytes) {
    if (!on) return (size_t)-1;
    const size_t at = nb;
    nb += (bytes + 15) / 16 * 16;
    return at;
  };
  const size_t v3 = sizeof(double) * 3 * (size_t)n_tot;
  const size_t o_pos = sec(true, v3), o_vel = sec(has_vel, v3), o_acel = sec(has_acel, v3),
               o_force = sec(has_force, v3), o_pold = sec(has_pold, v3),
               o_ocg = sec(has_ocg, v3), o_epot = sec(has_epot, sizeof(double) * n_tot),
               o_id = sec(has_id, sizeof(long long) * n_tot),
               o_z = sec(true, sizeof(int) * n_tot), o_rk = sec(true, sizeof(int) * n_tot),
               o_gk = sec(true, sizeof(int) * n_tot), o_off = sec(true, sizeof(int) * (nrep + 1)),
               o_skip = sec(has_skip, n_tot);
  // The device buffer has the section layout above.  Each replica's parts of
  // the sections are assembled in one half of a pinned buffer (pageable
  // copies are slow here) and sent while the next replica fills the other
  // half; an event guards a half until its copies have read it.
  cudaStream_t st = c->stream;
  unsigned char* db = nullptr;
  CK(cudaMalloc(&db, nb > 0 ? nb : 16));
  size_t per_atom = 24 + 12;  // pos; z, hs%ref and gcmc places
  for (bool on : {has_vel, has_acel, has_force, has_pold, has_ocg}) per_atom += on ? 24 : 0;
  per_atom += (has_epot ? 8 : 0) + (has_id ? 8 : 0) + (has_skip ? 1 : 0);
  int nmax = 0;
  for (int r = 0; r < nrep; ++r) nmax = std::max(nmax, atoms[r].n);
  const size_t half = (size_t)nmax * per_atom + 16 * 16;
  // host threads, each with its own slot of the pinned buffer and an event
  const int K = std::max(1, std::min({8, nrep, (int)std::thread::hardware_concurrency()}));
  cudaError_t e = cudaSuccess;
  if ((size_t)K * half > c->h_stage_bytes) {
    if (c->h_stage) cudaFreeHost(c->h_stage);
    c->h_stage = nullptr;
    c->h_stage_bytes = 0;
    e = cudaMallocHost(&c->h_stage, (size_t)K * half);
    if (e == cudaSuccess) c->h_stage_bytes = (size_t)K * half;
  }
  std::vector<cudaEvent_t> ev(K, nullptr);
  for (int t = 0; t < K && e == cudaSuccess; ++t) {
    e = cudaEventCreateWithFlags(&ev[t], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventRecord(ev[t], st);
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(db + o_off, off.data(), sizeof(int) * (nrep + 1), cudaMemcpyHostToDevice, st);
  std::memset(c->h_sc, 0, sizeof(Scalars) * nrep);
  const bool gcmc = c->P.reservoir == DML_RESERVOIR_GCMC;
  std::atomic<int> bad_z{0};
  std::vector<cudaError_t> terr(K, cudaSuccess);
  // thread t fills replicas t, t + K, ... into its slot (the slot's previous
  // copies are waited for first) and queues their copies on the stream
  // own: the thread was started here (the caller's thread keeps its device)
  auto worker = [&](int t, bool own) {
    cudaError_t& te = terr[t];
    te = own ? cudaSetDevice(c->device) : cudaSuccess;
    for (int r = t; r < nrep && te == cudaSuccess && !bad_z.load(); r += K) {
    const dml_atoms* a = atoms + r;
    const int n = a->n, o = off[r];
    te = cudaEventSynchronize(ev[t]);  // the slot's previous copies are done
    if (te != cudaSuccess) break;
    unsigned char* const base = static_cast<unsigned char*>(c->h_stage) + (size_t)t * half;
    size_t lo = 0;
    struct Part {
      size_t at, dst, bytes;
    };
    Part parts[16];
    int np = 0;
    // this replica's part of section sec_off (elem bytes per atom)
    auto part = [&](size_t sec_off, size_t elem) -> unsigned char* {
      if (sec_off == (size_t)-1) return nullptr;
      unsigned char* q = base + lo;
      parts[np++] = Part{lo, sec_off + elem * (size_t)o, elem * (size_t)n};
      lo += (elem * (size_t)n + 15) / 16 * 16;
      return q;
    };
    auto put3 = [&](size_t sec_off, const double* src, double def) {
      double* dst = reinterpret_cast<double*>(part(sec_off, 24));
      if (!dst) return;
      if (src) std::memcpy(dst, src, sizeof(double) * 3 * n);
      else std::fill(dst, dst + 3 * (size_t)n, def);
    };
    put3(o_pos, a->pos, 0.0);
    put3(o_vel, a->vel, 0.0);
    put3(o_acel, a->acel, 0.0);
    put3(o_force, a->force, 0.0);
    put3(o_pold, a->pos_old ? a->pos_old : a->pos, 0.0);  // pos_old defaults to pos
    put3(o_ocg, a->old_cg, 1e8);
    if (has_epot) {
      double* dst = reinterpret_cast<double*>(part(o_epot, 8));
      if (a->epot) std::memcpy(dst, a->epot, sizeof(double) * n);
      else std::fill(dst, dst + n, 0.0);
    }
    if (has_skip) {
      int8_t* dst = reinterpret_cast<int8_t*>(part(o_skip, 1));
      if (a->skip) std::memcpy(dst, a->skip, n);
      else std::memset(dst, 0, n);
    }
    int64_t max_id = n - 1;
    if (has_id) {
      long long* dst = reinterpret_cast<long long*>(part(o_id, 8));
      if (a->id) {
        max_id = -1;
        for (int i = 0; i < n; ++i) {
          dst[i] = a->id[i];
          max_id = std::max<int64_t>(max_id, a->id[i]);
        }
      } else {
        for (int i = 0; i < n; ++i) dst[i] = i;
      }
    }
    int* zd = reinterpret_cast<int*>(part(o_z, 4));
    int* rk = reinterpret_cast<int*>(part(o_rk, 4));
    int* gk = reinterpret_cast<int*>(part(o_gk, 4));
    int nref = 0, ng = 0;
    for (int i = 0; i < n; ++i) {
      const int z = a->z[i];
      if (z < 1 || z > 3) {
        bad_z.store(1);
        break;
      }
      zd[i] = z;
      // hs%ref holds the mobile atoms in sys order
      const bool in_ref = a->in_ref ? a->in_ref[i] != 0 : (z != DML_Z_CG);
      rk[i] = in_ref ? nref++ : -1;
      // gcmc attach loop (dana.F90:130-137): z == 1 atoms in sys order
      const bool gm = gcmc && (a->in_gcmc ? a->in_gcmc[i] != 0 : z == DML_Z_LI);
      gk[i] = gm ? ng++ : -1;
    }
    if (bad_z.load()) break;
    for (int k = 0; k < np && te == cudaSuccess; ++k)
      if (parts[k].bytes)
        te = cudaMemcpyAsync(db + parts[k].dst, base + parts[k].at, parts[k].bytes,
                             cudaMemcpyHostToDevice, st);
    if (te == cudaSuccess) te = cudaEventRecord(ev[t], st);
    Scalars& S = c->h_sc[r];
    S.zmax = c->reps[r].zmax;
    S.zmax_frame = S.zmax;
    S.z0 = c->reps[r].z0;
    S.z1 = c->reps[r].z1;
    S.n_slots = n;
    S.n_b = n;
    S.n_rank = nref;
    S.n_ref = nref;
    S.n_atoms = n;
    S.n_alist = n;
    S.n_gorder = ng;
    S.n_gcmc = ng;
    S.b_nat = n;
    S.nlimbo = 0;
    S.free_lo = n;  // slots are dense after loading
    S.bfree_lo = n;
    S.next_id = max_id + 1;
    // config_chunk: the template atoms take the next ids (never keys of a
    // draw: they do not move)
    if (c->P.reservoir == DML_RESERVOIR_CHUNKS) S.next_id += (long long)c->chunk_z.size();
    }
  };
  if (e == cudaSuccess) {
    std::vector<std::thread> th;
    int started = 1;
    try {
      for (; started < K; ++started) th.emplace_back(worker, started, true);
    } catch (...) {  // no more threads: the caller's thread takes the rest
    }
    worker(0, false);
    for (int t = started; t < K; ++t) worker(t, false);
    for (std::thread& x : th) x.join();
    for (int t = 0; t < K; ++t)
      if (e == cudaSuccess) e = terr[t];
  }
  // the pinned slots are read by the copies: wait for them before leaving
  {
    const cudaError_t e2 = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = e2;
  }
  for (cudaEvent_t x : ev)
    if (x) cudaEventDestroy(x);
  if (e != cudaSuccess || bad_z.load()) {
    cudaFree(db);
    if (bad_z.load()) return DML_E_ARG;
    return cuda_fail(c, e, "staged atom upload");
  }
  LoadIn in{};
  auto dp = [&](size_t o) -> const void* { return o == (size_t)-1 ? nullptr : db + o; };
  in.pos = static_cast<const double*>(dp(o_pos));
  in.vel = static_cast<const double*>(dp(o_vel));
  in.acel = static_cast<const double*>(dp(o_acel));
  in.force = static_cast<const double*>(dp(o_force));
  in.pos_old = static_cast<const double*>(dp(o_pold));
  in.old_cg = static_cast<const double*>(dp(o_ocg));
  in.epot = static_cast<const double*>(dp(o_epot));
  in.id = static_cast<const long long*>(dp(o_id));
  in.z = static_cast<const int*>(dp(o_z));
  in.rk = static_cast<const int*>(dp(o_rk));
  in.gk = static_cast<const int*>(dp(o_gk));
  in.off = static_cast<const int*>(dp(o_off));
  in.skip = static_cast<const int8_t*>(dp(o_skip));
  in.n_tot = n_tot;
  const char* what = "cudaMemsetAsync (index arrays)";
  // every index array of the layout starts at -1 (no atom, no slot)
  for (int* a : {d.rank, d.ref, d.bslot, d.b2hs, d.alist, d.apos, d.gorder, d.gpos})
    if (e == cudaSuccess) {
      what = "cudaMemsetAsync (index arrays)";
      e = cudaMemsetAsync(a, 0xFF, sizeof(int) * cap, st);
    }
  if (e == cudaSuccess) {
    what = "cudaMemcpyAsync (replica constants)";
    e = cudaMemcpyAsync(d.rc, c->rc.data(), sizeof(RepConst) * nrep, cudaMemcpyHostToDevice, st);
  }
  if (e == cudaSuccess) {
    what = "load_atoms_kernel launch";
    k_load_atoms(d, c->K, in, st);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && c->K.mixed) {  // loaded forces may be nonzero anywhere
    what = "cudaMemsetAsync (force bits)";
    e = cudaMemsetAsync(d.fnz, 0xFF, sizeof(unsigned) * ((size_t)d.cap / 32 + 1), st);
  }
  if (e == cudaSuccess) {
    what = "load_atoms_kernel";
    e = cudaStreamSynchronize(st);
  }
  cudaFree(db);
  if (e != cudaSuccess) return cuda_fail(c, e, what);
  CK(cudaMemcpyAsync(d.sc, c->h_sc, sizeof(Scalars) * nrep, cudaMemcpyHostToDevice, st));
  if (chunks) {
    // config_chunk (dana.F90:552-587): the template raised by zmax, its old
    // position by zmax again (as the reference writes it)
    std::vector<double4> tp((size_t)nrep * n_chunk), to((size_t)nrep * n_chunk);
    std::vector<int8_t> tz(n_chunk);
    for (int r = 0; r < nrep; ++r) {
      const double zm = c->reps[r].zmax;
      for (int j = 0; j < n_chunk; ++j) {
        const double* q = &c->chunk_pos[3 * (size_t)j];
        const double zr = q[2] + zm;
        tp[(size_t)r * n_chunk + j] = make_double4(q[0], q[1], zr, 0.0);
        to[(size_t)r * n_chunk + j] = make_double4(q[0], q[1], zr + zm, 0.0);
      }
    }
    for (int j = 0; j < n_chunk; ++j) tz[j] = (int8_t)c->chunk_z[j];
    CK(cudaMemcpyAsync(d.chk_pos, tp.data(), sizeof(double4) * tp.size(), cudaMemcpyHostToDevice,
                       st));
    CK(cudaMemcpyAsync(d.chk_pold, to.data(), sizeof(double4) * to.size(),
                       cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(d.chk_typ, tz.data(), tz.size(), cudaMemcpyHostToDevice, st));
    c->K.chunk_dist = c->chunk_dist;
    c->K.n_chunk = n_chunk;
  }
  // the context-wide state starts at zero but for the F members the load
  // listed for the first capture commit
  int n_f = 0;
  CK(cudaMemcpyAsync(&n_f, &d.g->n_f, sizeof n_f, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  std::memset(c->h_g, 0, sizeof(Global));
  c->h_g->n_f = n_f;
  CK(cudaMemcpyAsync(d.g, c->h_g, sizeof(Global), cudaMemcpyHostToDevice, st));
  CK(cudaStreamSynchronize(st));
  c->loaded = true;
  return 0;
}

int dml_set_atoms(dml_ctx* c, const dml_atoms* a) {
  if (!c || !a) return DML_E_ARG;
  if (c->D.nrep != 1) return DML_E_ARG;
  return dml_set_atoms_batch(c, a);
}

int dml_test_update(dml_ctx* c, int32_t* rebuilt) {
  if (!c || !c->loaded) return DML_E_STATE;
  k_rank_prefix(c->D, c->stream);  // rows in use of every replica
  k_test_update(c->D, c->K, c->D.cap, c->D.cap, c->D.cap, c->stream);
  int rc = finish(c);
  if (rc) return rc;
  if (rebuilt) {
    *rebuilt = 0;
    for (int r = 0; r < c->D.nrep; ++r) *rebuilt |= c->h_sc[r].rebuild;
  }
  return 0;
}

int dml_force(dml_ctx* c) {
  if (!c || !c->loaded) return DML_E_STATE;
  k_rank_prefix(c->D, c->stream);  // rows in use of every replica
  k_force_pairs(c->D, c->K, c->D.cap, false, c->stream);
  k_force_sum(c->D, c->K, c->D.cap, false, c->stream);
  return finish(c);
}

int dml_ermak_a(dml_ctx* c, int64_t step) {
  if (!c || !c->loaded) return DML_E_STATE;
  int rc = set_step(c, step);
  if (rc) return rc;
  k_ermak_a(c->D, c->K, c->D.cap, c->stream);
  return finish(c);
}

int dml_ermak_b(dml_ctx* c) {
  if (!c || !c->loaded) return DML_E_STATE;
  k_ermak_b(c->D, c->K, c->D.cap, c->stream);
  return finish(c);
}

int dml_brownian(dml_ctx* c, int64_t step) {
  if (!c || !c->loaded) return DML_E_STATE;
  int rc = set_step(c, step);
  if (rc) return rc;
  k_brownian(c->D, c->K, c->D.cap, c->stream);
  return finish(c);
}

int dml_overlap_moveback(dml_ctx* c, int64_t step) {
  if (!c || !c->loaded) return DML_E_STATE;
  int rc = set_step(c, step);
  if (rc) return rc;
  k_rank_prefix(c->D, c->stream);  // rows in use of every replica
  k_overlap(c->D, c->K, c->D.cap, c->D.cap, true, 2, c->stream);
  return finish(c);
}

int dml_capture_commit(dml_ctx* c, int32_t* n_new) {
  if (!c || !c->loaded) return DML_E_STATE;
  int zero = 0;
  for (int r = 0; r < c->D.nrep; ++r)
    CK(cudaMemcpyAsync(&c->D.sc[r].n_new_cg, &zero, sizeof zero, cudaMemcpyHostToDevice,
                       c->stream));
  k_capture_commit(c->D, c->K, c->D.cap, c->stream);
  int rc = finish(c);
  if (rc) return rc;
  if (n_new) {
    *n_new = 0;
    for (int r = 0; r < c->D.nrep; ++r) *n_new += c->h_sc[r].n_new_cg;
  }
  return 0;
}

int dml_gcmc(dml_ctx* c, int64_t step) {
  if (!c || !c->loaded) return DML_E_STATE;
  if (c->P.reservoir != DML_RESERVOIR_GCMC) return DML_E_RESERVOIR;
  int rc = set_step(c, step);
  if (rc) return rc;
  k_gcmc(c->D, c->K, c->D.cap, c->stream);
  return finish(c);
}

int dml_calc_rho(dml_ctx* c, double* rho) {
  if (!c || !c->loaded) return DML_E_STATE;
  k_calc_rho(c->D, c->K, c->D.cap, c->stream);
  int rc = finish(c);
  if (rc) return rc;
  if (rho) *rho = c->h_sc[0].rho;  // replica 0; every replica's rho in dml_get_counters_replica
  return 0;
}

int dml_piston(dml_ctx* c) {
  if (!c || !c->loaded) return DML_E_STATE;
  k_piston(c->D, c->K, c->D.cap, c->stream);
  return finish(c);
}

int dml_setup(dml_ctx* c) {
  if (!c || !c->loaded) return DML_E_STATE;
  int rc = dml_test_update(c, nullptr);
  if (rc) return rc;
  if (c->P.integrator == DML_INTEGRATOR_ERMAK) {
    rc = dml_force(c);
    if (rc) return rc;
  }
  rc = dml_calc_rho(c, nullptr);
  if (rc) return rc;
  for (int r = 0; r < c->D.nrep; ++r) c->h_sc[r].rho0 = c->h_sc[r].rho;  // rho0 (dana.F90:146)
  rc = write_scalars(c);
  if (rc) return rc;
  c->setup_done = true;
  return 0;
}

int dml_set_chunk(dml_ctx* c, int32_t n, const double* pos, const int32_t* z, double dist) {
  if (!c || n <= 0 || !pos || !z || !(dist > 0)) return DML_E_ARG;
  if (c->P.reservoir != DML_RESERVOIR_CHUNKS) return DML_E_RESERVOIR;
  if (c->loaded) return DML_E_STATE;
  for (int j = 0; j < n; ++j)
    if (z[j] < 1 || z[j] > 3) return DML_E_ARG;
  c->chunk_pos.assign(pos, pos + 3 * (size_t)n);
  c->chunk_z.assign(z, z + n);
  c->chunk_dist = dist;
  return 0;
}

int dml_bloques(dml_ctx* c) {
  if (!c || !c->loaded) return DML_E_STATE;
  if (c->P.reservoir != DML_RESERVOIR_CHUNKS) return DML_E_RESERVOIR;
  CK(cudaMemsetAsync(&c->D.g->chunk_event, 0, sizeof(int), c->stream));
  int nb = 0, nbody = 0;
  int rc = queue_bloques(c, false, &nb, &nbody);
  if (rc) return rc;
  return finish(c);
}

int dml_step_async(dml_ctx* c, int64_t nsteps) {
  if (!c || !c->loaded || !c->setup_done) return DML_E_STATE;
  return queue_steps(c, nsteps);
}

int dml_set_graph_steps(dml_ctx* c, int32_t k) {
  if (!c || k < 1) return DML_E_ARG;
  if (k != c->graph_steps && c->multi_graph) {
    CK(cudaStreamSynchronize(c->stream));
    cudaGraphExecDestroy(c->multi_graph);
    c->multi_graph = nullptr;
  }
  c->graph_steps = k;
  return 0;
}

int dml_time_run(dml_ctx* c, int64_t nsteps, double* ms) {
  if (!c || !ms || nsteps <= 0) return DML_E_ARG;
  if (!c->loaded || !c->setup_done) return DML_E_STATE;
  int rc = build_step_graph(c);
  if (!rc && c->graph_steps > 1 && nsteps >= c->graph_steps) rc = build_multi_graph(c);
  if (rc) return rc;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaStreamSynchronize(c->stream));
  CK(cudaEventRecord(e0, c->stream));
  rc = queue_steps(c, nsteps);
  CK(cudaEventRecord(e1, c->stream));
  CK(cudaEventSynchronize(e1));
  float t = 0;
  CK(cudaEventElapsedTime(&t, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  *ms = t;
  return finish(c);
}

int dml_sync(dml_ctx* c) {
  if (!c) return DML_E_ARG;
  return finish(c);
}

int dml_step(dml_ctx* c, int64_t nsteps) {
  int rc = dml_step_async(c, nsteps);
  if (rc) return rc;
  return finish(c);
}

int dml_time_steps(dml_ctx* c, int64_t nsteps, int32_t flush_l2, double* ms) {
  if (!c || !ms || nsteps <= 0) return DML_E_ARG;
  if (!c->loaded || !c->setup_done) return DML_E_STATE;
  int rc = build_step_graph(c);
  if (rc) return rc;
  scan_refresh(c);
  if (flush_l2 && (rc = ensure_flush(c)) != 0) return rc;
  std::vector<cudaEvent_t> ev(2 * nsteps);
  for (auto& e : ev) CK(cudaEventCreate(&e));
  for (int64_t i = 0; i < nsteps; ++i) {
    if (flush_l2) k_flush(c->flush_buf, kFlushBytes, c->stream);
    CK(cudaEventRecord(ev[2 * i], c->stream));
    CK(cudaGraphLaunch(c->step_graph, c->stream));
    CK(cudaEventRecord(ev[2 * i + 1], c->stream));
  }
  CK(cudaStreamSynchronize(c->stream));
  double tot = 0;
  for (int64_t i = 0; i < nsteps; ++i) {
    float t = 0;
    CK(cudaEventElapsedTime(&t, ev[2 * i], ev[2 * i + 1]));
    tot += t;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  *ms = tot;
  return finish(c);
}

int dml_profile_steps(dml_ctx* c, int64_t nsteps, int32_t flush_l2, double* phase_ms,
                      int32_t nphase) {
  if (!c || !phase_ms || nsteps <= 0 || nphase < DML_NPHASE) return DML_E_ARG;
  if (!c->loaded || !c->setup_done) return DML_E_STATE;
  int rc = 0;
  if (flush_l2 && (rc = ensure_flush(c)) != 0) return rc;
  const int ne = DML_NPHASE + 1;
  std::vector<cudaEvent_t> ev(ne * nsteps);
  for (auto& e : ev) CK(cudaEventCreate(&e));
  std::vector<ProfileGap> gaps;
  scan_refresh(c);
  for (int64_t i = 0; i < nsteps; ++i) {
    if (flush_l2) k_flush(c->flush_buf, kFlushBytes, c->stream);
    rc = enqueue_step(c, &ev[ne * i], false, nullptr, nullptr, &gaps);
    if (rc) return rc;
  }
  CK(cudaStreamSynchronize(c->stream));
  for (int k = 0; k < nphase; ++k) phase_ms[k] = 0;
  for (int64_t i = 0; i < nsteps; ++i)
    for (int k = 0; k < DML_NPHASE; ++k) {
      float t = 0;
      CK(cudaEventElapsedTime(&t, ev[ne * i + k], ev[ne * i + k + 1]));
      phase_ms[k] += t;
    }
  for (auto& gp : gaps) {
    float t = 0;
    CK(cudaEventElapsedTime(&t, gp.a, gp.b));
    phase_ms[gp.phase] -= t;
    cudaEventDestroy(gp.a);
    cudaEventDestroy(gp.b);
  }
  for (auto& e : ev) cudaEventDestroy(e);
  return finish(c);
}

// The chosen form's cells (no counterpart in the reference, whose cells
// are int(box / (rc + skin)) per axis): cells with an edge bound of
// factor * (rc + skin).  The lists hold the same atoms in another order (the
// 27-cell stencil still covers rc + skin), which the order-independent
// fixed-point sums do not see; overlap_moveback's examination order and
// gcmc_run's own-list order follow the list, so trajectories differ from
// factor 1 the way two seeds do.  Every list is rebuilt at the next
// test_update.  Cells are allocated for factor 1, so any factor >= 1 fits.
int dml_set_cell_factor(dml_ctx* c, double factor) {
  if (!c || !(factor >= 1.0 && factor <= 2.0)) return DML_E_ARG;
  if (!c->loaded) return DML_E_STATE;
  if (c->P.precision != DML_PRECISION_MIXED || c->P.reservoir == DML_RESERVOIR_CHUNKS)
    return DML_E_UNSUPPORTED;
  CK(cudaStreamSynchronize(c->stream));
  int rc = read_scalars(c);
  if (rc) return rc;
  Dev& d = c->D;
  int any_thread = 0, any_warp = 0;
  for (int r = 0; r < d.nrep; ++r) {
    RepConst& R = c->rc[r];
    RepConst T;
    make_repconst(c->P, c->reps[r], T, factor);
    if (!T.use_cells || !R.use_cells) continue;  // the all-pairs build keeps its path
    // the grid of the new factor; placement, capacity and margins stay
    for (int k = 0; k < 3; ++k) {
      R.ncells[k] = T.ncells[k];
      R.cell[k] = T.cell[k];
      R.inv_cellf[k] = T.inv_cellf[k];
      R.cellf[k] = T.cellf[k];
      R.head_dim[k] = T.head_dim[k];
    }
    R.ncell = T.ncell;
    R.tess_hif = T.tess_hif;
    R.gl_all = T.gl_all;
    R.gl_mask = T.gl_mask;
    R.gl_cmask = T.gl_cmask;
    const double cells = (double)R.ncells[0] * R.ncells[1] * R.ncells[2];
    R.list_thread = 27.0 * c->h_sc[r].n_b / cells <= kThreadRowCand ? 1 : 0;
    c->h_sc[r].listed = 0;
  }
  for (int r = 0; r < d.nrep; ++r) {
    if (!c->rc[r].use_cells) continue;
    if (c->rc[r].list_thread) any_thread = 1; else any_warp = 1;
  }
  if (any_thread != d.any_list_thread || any_warp != d.any_list_warp) {
    // the step graph launches the list builds in use: capture it again
    d.any_list_thread |= any_thread;
    d.any_list_warp |= any_warp;
    if (c->step_graph) cudaGraphExecDestroy(c->step_graph);
    if (c->multi_graph) cudaGraphExecDestroy(c->multi_graph);
    c->step_graph = nullptr;
    c->multi_graph = nullptr;
  }
  CK(cudaMemcpyAsync(d.rc, c->rc.data(), sizeof(RepConst) * d.nrep, cudaMemcpyHostToDevice,
                     c->stream));
  rc = write_scalars(c);
  if (rc) return rc;
  c->cell_factor = factor;
  return 0;
}

// Tries the cell factors 1.0, 1.1, .. 1.5: after each one's rebuild step,
// `steps` steps are timed, and the fastest factor is kept (its lists are
// rebuilt once more).  The run advances by kCellFactors * (steps + 1) + 1
// steps.
int dml_tune_cells(dml_ctx* c, int32_t steps, double* best) {
  if (!c || steps < 1) return DML_E_ARG;
  if (!c->loaded || !c->setup_done) return DML_E_STATE;
  double best_f = 1.0;
  float best_t = 1e30f;
  for (int v = 0; v < kCellFactors; ++v) {
    const double f = 1.0 + 0.1 * v;
    int rc = dml_set_cell_factor(c, f);
    if (rc) return rc;
    if ((rc = dml_step(c, 1)) != 0) return rc;  // the rebuild
    double ms = 0.0;
    if ((rc = dml_time_run(c, steps, &ms)) != 0) return rc;
    c->cell_us[v] = (float)(1e3 * ms / steps);
    if (c->cell_us[v] < best_t) {
      best_t = c->cell_us[v];
      best_f = f;
    }
  }
  int rc = dml_set_cell_factor(c, best_f);
  if (rc) return rc;
  if ((rc = dml_step(c, 1)) != 0) return rc;
  if (best) *best = best_f;
  return 0;
}

int dml_get_cell_tuning(dml_ctx* c, double* factor, float* us) {
  if (!c) return DML_E_ARG;
  if (factor) *factor = c->cell_factor;
  if (us)
    for (int v = 0; v < kCellFactors; ++v) us[v] = c->cell_us[v];
  return 0;
}

int dml_get_tuning(dml_ctx* c, int32_t* scan_lanes, float* scan_us) {
  if (!c) return DML_E_ARG;
  if (scan_lanes)
    *scan_lanes = c->P.integrator == DML_INTEGRATOR_ERMAK ? c->K.scan_lanes : c->K.near_lanes;
  if (scan_us)
    for (int v = 0; v < kScanMappings; ++v) scan_us[v] = c->tune_us[v];
  return 0;
}

int dml_check_conversions(const double* x, int64_t n, float* f32, double* back) {
  if (n < 0 || (n > 0 && (!x || !f32 || !back))) return DML_E_ARG;
  if (n == 0) return 0;
  double *dx = nullptr, *db = nullptr;
  float* df = nullptr;
  cudaError_t e = cudaMalloc(&dx, sizeof(double) * n);
  if (e == cudaSuccess) e = cudaMalloc(&db, sizeof(double) * n);
  if (e == cudaSuccess) e = cudaMalloc(&df, sizeof(float) * n);
  if (e == cudaSuccess) e = cudaMemcpy(dx, x, sizeof(double) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    k_check_conversions(dx, df, db, n, 0);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(f32, df, sizeof(float) * n, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(back, db, sizeof(double) * n, cudaMemcpyDeviceToHost);
  cudaFree(dx);
  cudaFree(db);
  cudaFree(df);
  return e == cudaSuccess ? 0 : DML_E_CUDA;
}

int dml_check_normals(const uint32_t* words, int64_t n_pairs, int32_t precision, float* out) {
  if (n_pairs < 0 || (n_pairs > 0 && (!words || !out))) return DML_E_ARG;
  if (precision != DML_PRECISION_FP64 && precision != DML_PRECISION_MIXED) return DML_E_ARG;
  if (n_pairs == 0) return 0;
  unsigned* dw = nullptr;
  float* dout = nullptr;
  cudaError_t e = cudaMalloc(&dw, sizeof(unsigned) * 2 * n_pairs);
  if (e == cudaSuccess) e = cudaMalloc(&dout, sizeof(float) * 2 * n_pairs);
  if (e == cudaSuccess)
    e = cudaMemcpy(dw, words, sizeof(unsigned) * 2 * n_pairs, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    k_check_normals(dw, dout, n_pairs, precision == DML_PRECISION_MIXED ? 1 : 0, 0);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpy(out, dout, sizeof(float) * 2 * n_pairs, cudaMemcpyDeviceToHost);
  cudaFree(dw);
  cudaFree(dout);
  return e == cudaSuccess ? 0 : DML_E_CUDA;
}

int dml_check_pick(const uint64_t* k, const int32_t* n, int64_t count, int32_t* m) {
  if (count < 0 || (count > 0 && (!k || !n || !m))) return DML_E_ARG;
  if (count == 0) return 0;
  unsigned long long* dk = nullptr;
  int *dn = nullptr, *dm = nullptr;
  cudaError_t e = cudaMalloc(&dk, sizeof(unsigned long long) * count);
  if (e == cudaSuccess) e = cudaMalloc(&dn, sizeof(int) * count);
  if (e == cudaSuccess) e = cudaMalloc(&dm, sizeof(int) * count);
  if (e == cudaSuccess) e = cudaMemcpy(dk, k, sizeof(unsigned long long) * count, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dn, n, sizeof(int) * count, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    k_check_pick(dk, dn, dm, count, 0);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(m, dm, sizeof(int) * count, cudaMemcpyDeviceToHost);
  cudaFree(dk);
  cudaFree(dn);
  cudaFree(dm);
  return e == cudaSuccess ? 0 : DML_E_CUDA;
}

int dml_launches_per_step(dml_ctx* c, int32_t* per_rebuild) {
  if (!c) return -DML_E_ARG;
  if (!c->launches_per_step) {
    int rc = build_step_graph(c);
    if (rc) return -rc;
  }
  if (per_rebuild) *per_rebuild = c->launches_per_rebuild;
  return c->launches_per_step;
}

int dml_get_counters_replica(dml_ctx* c, int32_t rep, dml_counters* o) {
  if (!c || !o || rep < 0 || rep >= c->D.nrep) return DML_E_ARG;
  std::memset(o, 0, sizeof *o);
  if (!c->loaded) return 0;
  int rc = read_scalars(c);
  if (rc) return rc;
  const Scalars& s = c->h_sc[rep];
  o->try_ = (int64_t)s.try_;
  o->depo = (int64_t)s.depo;
  o->choques = (int64_t)s.choques;
  o->choques3 = (int64_t)s.choques3;
  o->nupd = (int64_t)s.nupd;
  o->step = c->h_g->step;
  o->list_builds = c->h_g->list_builds;
  o->gcmc_ins = (int64_t)s.gcmc_ins;
  o->gcmc_del = (int64_t)s.gcmc_del;
  o->n_atoms = s.n_atoms;
  o->n_ref = s.n_ref;
  o->max_nn = s.max_nn;
  o->passes = s.passes;
  o->zmax = s.zmax;
  o->z0 = s.z0;
  o->rho = s.rho;
  o->rho0 = s.rho0;
  return 0;
}

int dml_get_scan_counts(dml_ctx* c, int32_t rep, int64_t* full, int64_t* partial) {
  if (!c || rep < 0 || rep >= c->D.nrep) return DML_E_ARG;
  Scalars v;
  std::memset(&v, 0, sizeof v);
  if (c->loaded) {
    CK(cudaMemcpyAsync(&v, c->D.sc + rep, sizeof v, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  if (full) *full = (int64_t)v.sl_nfull;
  if (partial) *partial = (int64_t)v.sl_npartial;
  return 0;
}

int dml_get_test_counts(dml_ctx* c, int32_t rep, int64_t* tests, int64_t* exact) {
  if (!c || rep < 0 || rep >= c->D.nrep) return DML_E_ARG;
  Scalars v;
  std::memset(&v, 0, sizeof v);
  if (c->loaded) {
    CK(cudaMemcpyAsync(&v, c->D.sc + rep, sizeof v, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  if (tests) *tests = (int64_t)v.dt_tests;
  if (exact) *exact = (int64_t)v.dt_exact;
  return 0;
}

int dml_set_scan_lanes(dml_ctx* c, int32_t lanes) {
  if (!c || !(lanes == 0 || lanes == 1 || lanes == 2 || lanes == 4 || lanes == 8 ||
              lanes == 16 || lanes == 32))
    return DML_E_ARG;
  c->forced_lanes = lanes;
  if (c->step_graph || c->multi_graph) {
    CK(cudaStreamSynchronize(c->stream));
    if (c->step_graph) cudaGraphExecDestroy(c->step_graph);
    if (c->multi_graph) cudaGraphExecDestroy(c->multi_graph);
    c->step_graph = nullptr;
    c->multi_graph = nullptr;
  }
  return 0;
}

int dml_get_gcmc_paths(dml_ctx* c, int32_t rep, int64_t* parallel, int64_t* sequential) {
  if (!c || rep < 0 || rep >= c->D.nrep) return DML_E_ARG;
  int v[kCntStride] = {0};
  if (c->loaded) {
    CK(cudaMemcpyAsync(v, c->D.pr_cnt + (size_t)rep * kCntStride, sizeof v,
                       cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  if (parallel) *parallel = v[kCntGcmcPar];
  if (sequential) *sequential = v[kCntGcmcSeq];
  return 0;
}

// Sums over replicas for the event counters and atom counts; the geometry
// (zmax, z0, rho, rho0) is replica 0's, max_nn and passes the maxima.
int dml_get_counters(dml_ctx* c, dml_counters* o) {
  if (!c || !o) return DML_E_ARG;
  int rc = dml_get_counters_replica(c, 0, o);
  if (rc || !c->loaded) return rc;
  for (int r = 1; r < c->D.nrep; ++r) {
    const Scalars& s = c->h_sc[r];
    o->try_ += (int64_t)s.try_;
    o->depo += (int64_t)s.depo;
    o->choques += (int64_t)s.choques;
    o->choques3 += (int64_t)s.choques3;
    o->nupd += (int64_t)s.nupd;
    o->gcmc_ins += (int64_t)s.gcmc_ins;
    o->gcmc_del += (int64_t)s.gcmc_del;
    o->n_atoms += s.n_atoms;
    o->n_ref += s.n_ref;
    o->max_nn = std::max(o->max_nn, s.max_nn);
    o->passes = std::max(o->passes, s.passes);
  }
  return 0;
}

// salida resets try and depo after each output (dana.F90:252-258).
int dml_reset_counters(dml_ctx* c) {
  if (!c || !c->loaded) return DML_E_STATE;
  int rc = read_scalars(c);
  if (rc) return rc;
  for (int r = 0; r < c->D.nrep; ++r) c->h_sc[r].try_ = c->h_sc[r].depo = 0;
  return write_scalars(c);
}

// Replica `rep`'s atoms in sys%alist order (its slots are [base, base + cap)).
int dml_get_atoms_replica(dml_ctx* c, int32_t rep, dml_atoms* a) {
  if (!c || !a || rep < 0 || rep >= c->D.nrep) return DML_E_ARG;
  if (!c->loaded) return DML_E_STATE;
  int rc = read_scalars(c);
  if (rc) return rc;
  const int B = c->rc[rep].base;
  const int ns = c->h_sc[rep].n_slots, nal = c->h_sc[rep].n_alist;
  const Dev& d = c->D;
  cudaStream_t s = c->stream;
  // One pinned buffer holds the sys%alist segment and the requested fields
  // (16-byte aligned sections, uninitialised: every byte read is copied in).
  const bool want_vel = a->vel || a->acel;
  const bool want_acel = a->acel && !c->K.mixed;
  size_t nb = 0;
  auto sec = [&](bool on, size_t bytes) {
    const size_t at = nb;
    if (on) nb += (bytes + 15) / 16 * 16;
    return at;
  };
  const size_t o_al = sec(true, sizeof(int) * nal), o_pos = sec(a->pos, sizeof(double4) * ns),
               o_vel = sec(want_vel, sizeof(double4) * ns),
               o_acel = sec(want_acel, sizeof(double4) * ns),
               o_force = sec(a->force, sizeof(double4) * ns),
               o_pold = sec(a->pos_old, sizeof(double4) * ns),
               o_ocg = sec(a->old_cg, sizeof(double4) * ns),
               o_epot = sec(a->epot, sizeof(double) * ns), o_typ = sec(a->z, ns),
               o_skip = sec(a->skip, ns), o_ing = sec(a->in_gcmc, ns),
               o_id = sec(a->id, sizeof(long long) * ns), o_rank = sec(a->in_ref, sizeof(int) * ns);
  if (nb > c->h_stage_bytes) {
    if (c->h_stage) cudaFreeHost(c->h_stage);
    c->h_stage = nullptr;
    c->h_stage_bytes = 0;
    CK(cudaMallocHost(&c->h_stage, nb + nb / 4));
    c->h_stage_bytes = nb + nb / 4;
  }
  char* const hs = static_cast<char*>(c->h_stage);
  const int* alist = reinterpret_cast<const int*>(hs + o_al);
  const double4* pos = reinterpret_cast<const double4*>(hs + o_pos);
  const double4* vel = reinterpret_cast<const double4*>(hs + o_vel);
  const double4* acel = reinterpret_cast<const double4*>(hs + o_acel);
  const double4* force = reinterpret_cast<const double4*>(hs + o_force);
  const double4* pos_old = reinterpret_cast<const double4*>(hs + o_pold);
  const double4* old_cg = reinterpret_cast<const double4*>(hs + o_ocg);
  const double* epot = reinterpret_cast<const double*>(hs + o_epot);
  const int8_t* typ = reinterpret_cast<const int8_t*>(hs + o_typ);
  const int8_t* skip = reinterpret_cast<const int8_t*>(hs + o_skip);
  const int8_t* ing = reinterpret_cast<const int8_t*>(hs + o_ing);
  const long long* id = reinterpret_cast<const long long*>(hs + o_id);
  const int* rank = reinterpret_cast<const int*>(hs + o_rank);
  if (nal)
    CK(cudaMemcpyAsync(hs + o_al, d.alist + B, sizeof(int) * nal, cudaMemcpyDeviceToHost, s));
  auto get = [&](size_t off, const void* src, size_t elem) -> cudaError_t {
    if (!ns) return cudaSuccess;
    return cudaMemcpyAsync(hs + off, (const char*)src + elem * B, elem * ns, cudaMemcpyDeviceToHost, s);
  };
  // only the fields asked for travel (NULL outputs are skipped)
  if (a->pos) CK(get(o_pos, d.pos, sizeof(double4)));
  if (want_vel) CK(get(o_vel, d.vel, sizeof(double4)));
  if (want_acel) CK(get(o_acel, d.acel, sizeof(double4)));
  if (a->force) CK(get(o_force, d.force, sizeof(double4)));
  if (a->pos_old) CK(get(o_pold, d.pos_old, sizeof(double4)));
  if (a->old_cg) CK(get(o_ocg, d.old_cg, sizeof(double4)));
  if (a->epot) CK(get(o_epot, d.epot, sizeof(double)));
  if (a->z) CK(get(o_typ, d.typ, 1));
  if (a->skip) CK(get(o_skip, d.skip, 1));
  if (a->in_gcmc) CK(get(o_ing, d.in_gcmc, 1));
  if (a->id) CK(get(o_id, d.id, sizeof(long long)));
  if (a->in_ref) CK(get(o_rank, d.rank, sizeof(int)));
  CK(cudaStreamSynchronize(s));
  int n = 0;
  for (int q = 0; q < nal; ++q)
    if (alist[q] >= 0) ++n;
  if (a->n < n) return DML_E_ARG;
  a->n = n;
  int i = 0;
  for (int q = 0; q < nal; ++q) {
    int h = alist[q] - B;
    if (alist[q] < 0) continue;
    if (h < 0 || h >= ns) return DML_E_STATE;
    auto put = [&](double* dst, const double4& v) {
      if (!dst) return;
      dst[3 * i] = v.x;
      dst[3 * i + 1] = v.y;
      dst[3 * i + 2] = v.z;
    };
    // a section is read only when its field was requested (and copied)
    if (a->pos) put(a->pos, pos[h]);
    if (want_vel && c->K.mixed) {
      const float4 v = unpack_f3(vel[h]);
      const float4 ac = unpack_f3(make_double4(vel[h].z, vel[h].w, 0.0, 0.0));
      put(a->vel, make_double4(v.x, v.y, v.z, 0.0));
      put(a->acel, make_double4(ac.x, ac.y, ac.z, 0.0));
    } else if (want_vel) {
      put(a->vel, vel[h]);
      if (want_acel) put(a->acel, acel[h]);
    }
    if (a->force) put(a->force, force[h]);
    if (a->pos_old) put(a->pos_old, pos_old[h]);
    if (a->old_cg) put(a->old_cg, old_cg[h]);
    if (a->epot) a->epot[i] = epot[h];
    if (a->z) a->z[i] = typ[h];
    if (a->skip) a->skip[i] = skip[h];
    if (a->in_ref) a->in_ref[i] = rank[h] >= 0 ? 1 : 0;
    if (a->in_gcmc) a->in_gcmc[i] = ing[h];
    if (a->id) a->id[i] = id[h];
    ++i;
  }
  return 0;
}

// salida (dana.F90:1143-1183): one kernel writes every replica's record
// and zeroes try and depo on the device.
int dml_salida(dml_ctx* c, dml_observables* out) {
  if (!c || !out) return DML_E_ARG;
  if (!c->loaded) return DML_E_STATE;
  const int nrep = c->D.nrep;
  if (!c->d_obs) CK(cudaMalloc(&c->d_obs, sizeof(dml_observables) * nrep));
  k_salida(c->D, c->K, c->P.kb_driver, c->d_obs, c->stream);
  CK(cudaMemcpyAsync(out, c->d_obs, sizeof(dml_observables) * nrep, cudaMemcpyDeviceToHost,
                     c->stream));
  return finish(c);
}

int dml_get_atom_counts(dml_ctx* c, int32_t* out) {
  if (!c || !out) return DML_E_ARG;
  if (!c->loaded) return DML_E_STATE;
  int rc = read_scalars(c);
  if (rc) return rc;
  for (int r = 0; r < c->D.nrep; ++r) out[r] = c->h_sc[r].n_atoms;
  return 0;
}

int dml_get_atoms_batch(dml_ctx* c, dml_atoms* atoms) {
  if (!c || !atoms) return DML_E_ARG;
  if (!c->loaded) return DML_E_STATE;
  const int nrep = c->D.nrep;
  const dml_atoms& a0 = atoms[0];
  auto same = [&](const dml_atoms& a) {
    return !a.pos == !a0.pos && !a.vel == !a0.vel && !a.acel == !a0.acel &&
           !a.force == !a0.force && !a.pos_old == !a0.pos_old && !a.old_cg == !a0.old_cg &&
           !a.epot == !a0.epot && !a.z == !a0.z && !a.skip == !a0.skip &&
           !a.in_ref == !a0.in_ref && !a.in_gcmc == !a0.in_gcmc && !a.id == !a0.id;
  };
  for (int r = 0; r < nrep; ++r)
    if (!same(atoms[r])) return DML_E_ARG;
  int rc = read_scalars(c);
  if (rc) return rc;
  std::vector<long long> off(nrep + 1, 0);
  for (int r = 0; r < nrep; ++r) {
    if (atoms[r].n < c->h_sc[r].n_atoms) return DML_E_ARG;
    off[r + 1] = off[r] + c->h_sc[r].n_atoms;
  }
  const long long tot = off[nrep];
  // device sections, 16-byte aligned: the packed members, the offsets, the error word
  size_t nb = 0;
  auto sec = [&](bool on, size_t bytes) {
    const size_t at = nb;
    if (on) nb += (bytes + 15) / 16 * 16;
    return at;
  };
  const size_t v3 = sizeof(double) * 3 * (size_t)tot;
  const size_t o_pos = sec(a0.pos, v3), o_vel = sec(a0.vel, v3), o_acel = sec(a0.acel, v3),
               o_force = sec(a0.force, v3), o_pold = sec(a0.pos_old, v3),
               o_ocg = sec(a0.old_cg, v3), o_epot = sec(a0.epot, sizeof(double) * tot),
               o_z = sec(a0.z, sizeof(int) * tot), o_skip = sec(a0.skip, tot),
               o_inref = sec(a0.in_ref, tot), o_ing = sec(a0.in_gcmc, tot),
               o_id = sec(a0.id, sizeof(long long) * tot),
               o_off = sec(true, sizeof(long long) * (nrep + 1)), o_err = sec(true, sizeof(int));
  if (nb > c->d_stage_bytes) {
    if (c->d_stage) cudaFree(c->d_stage);
    c->d_stage = nullptr;
    c->d_stage_bytes = 0;
    CK(cudaMalloc(&c->d_stage, nb + nb / 4));
    c->d_stage_bytes = nb + nb / 4;
  }
  char* const ds = static_cast<char*>(c->d_stage);
  cudaStream_t s = c->stream;
  PackOut o{};
  auto dp = [&](bool on, size_t at) -> void* { return on ? ds + at : nullptr; };
  o.pos = static_cast<double*>(dp(a0.pos, o_pos));
  o.vel = static_cast<double*>(dp(a0.vel, o_vel));
  o.acel = static_cast<double*>(dp(a0.acel, o_acel));
  o.force = static_cast<double*>(dp(a0.force, o_force));
  o.pos_old = static_cast<double*>(dp(a0.pos_old, o_pold));
  o.old_cg = static_cast<double*>(dp(a0.old_cg, o_ocg));
  o.epot = static_cast<double*>(dp(a0.epot, o_epot));
  o.z = static_cast<int*>(dp(a0.z, o_z));
  o.skip = static_cast<int8_t*>(dp(a0.skip, o_skip));
  o.in_ref = static_cast<int8_t*>(dp(a0.in_ref, o_inref));
  o.in_gcmc = static_cast<int8_t*>(dp(a0.in_gcmc, o_ing));
  o.id = static_cast<long long*>(dp(a0.id, o_id));
  o.off = reinterpret_cast<const long long*>(ds + o_off);
  o.err = reinterpret_cast<int*>(ds + o_err);
  CK(cudaMemcpyAsync(ds + o_off, off.data(), sizeof(long long) * (nrep + 1),
                     cudaMemcpyHostToDevice, s));
  CK(cudaMemsetAsync(ds + o_err, 0, sizeof(int), s));
  (void)cudaGetLastError();  // an error left by an earlier caller (the slot is shared)
  k_pack_atoms(c->D, c->K, o, s);
  CK(cudaGetLastError());
  // The callers' arrays (pageable memory, where a direct device copy is
  // slow): each replica's members travel to one half of a pinned buffer
  // while the previous replica's half is copied out on the host.
  struct Mem {
    bool on;
    size_t at, elem;
  };
  const Mem mem[12] = {{a0.pos != nullptr, o_pos, 24},   {a0.vel != nullptr, o_vel, 24},
                       {a0.acel != nullptr, o_acel, 24}, {a0.force != nullptr, o_force, 24},
                       {a0.pos_old != nullptr, o_pold, 24}, {a0.old_cg != nullptr, o_ocg, 24},
                       {a0.epot != nullptr, o_epot, 8},  {a0.z != nullptr, o_z, 4},
                       {a0.skip != nullptr, o_skip, 1},  {a0.in_ref != nullptr, o_inref, 1},
                       {a0.in_gcmc != nullptr, o_ing, 1}, {a0.id != nullptr, o_id, 8}};
  size_t per_atom = 0;
  for (const Mem& m : mem)
    if (m.on) per_atom += m.elem;
  long long nmax = 0;
  for (int r = 0; r < nrep; ++r) nmax = std::max(nmax, off[r + 1] - off[r]);
  const size_t half = ((size_t)nmax * per_atom + 15) / 16 * 16 + 16 * 12;
  // host threads, each with its own slot of the pinned buffer and an event:
  // thread t copies replicas t, t + K, ... through its slot
  const int K = std::max(1, std::min({8, nrep, (int)std::thread::hardware_concurrency()}));
  if ((size_t)K * half > c->h_stage_bytes) {
    if (c->h_stage) cudaFreeHost(c->h_stage);
    c->h_stage = nullptr;
    c->h_stage_bytes = 0;
    CK(cudaMallocHost(&c->h_stage, (size_t)K * half));
    c->h_stage_bytes = (size_t)K * half;
  }
  std::vector<cudaEvent_t> ev(K, nullptr);
  cudaError_t e = cudaSuccess;
  for (int t = 0; t < K && e == cudaSuccess; ++t)
    e = cudaEventCreateWithFlags(&ev[t], cudaEventDisableTiming);
  auto dst_of = [&](const dml_atoms& a, int k) -> void* {
    void* const p[12] = {a.pos, a.vel, a.acel, a.force, a.pos_old, a.old_cg,
                         a.epot, a.z, a.skip, a.in_ref, a.in_gcmc, a.id};
    return p[k];
  };
  std::vector<cudaError_t> terr(K, cudaSuccess);
  // own: the thread was started here (the caller's thread keeps its device)
  auto worker = [&](int t, bool own) {
    cudaError_t& te = terr[t];
    te = own ? cudaSetDevice(c->device) : cudaSuccess;
    unsigned char* const hs = static_cast<unsigned char*>(c->h_stage) + (size_t)t * half;
    for (int r = t; r < nrep && te == cudaSuccess; r += K) {
      const size_t n = (size_t)(off[r + 1] - off[r]), b = (size_t)off[r];
      if (!n) continue;
      size_t at = 0;
      for (const Mem& m : mem) {
        if (!m.on) continue;
        if (te == cudaSuccess)
          te = cudaMemcpyAsync(hs + at, ds + m.at + m.elem * b, m.elem * n, cudaMemcpyDeviceToHost, s);
        at += (m.elem * n + 15) / 16 * 16;
      }
      if (te == cudaSuccess) te = cudaEventRecord(ev[t], s);
      if (te == cudaSuccess) te = cudaEventSynchronize(ev[t]);
      if (te != cudaSuccess) break;
      at = 0;
      for (int k = 0; k < 12; ++k) {
        if (!mem[k].on) continue;
        std::memcpy(dst_of(atoms[r], k), hs + at, mem[k].elem * n);
        at += (mem[k].elem * n + 15) / 16 * 16;
      }
    }
  };
  if (e == cudaSuccess) {
    std::vector<std::thread> th;
    int started = 1;
    try {
      for (; started < K; ++started) th.emplace_back(worker, started, true);
    } catch (...) {  // no more threads: the caller's thread takes the rest
    }
    worker(0, false);
    for (int t = started; t < K; ++t) worker(t, false);
    for (std::thread& x : th) x.join();
    for (int t = 0; t < K; ++t)
      if (e == cudaSuccess) e = terr[t];
  }
  for (cudaEvent_t x : ev)
    if (x) cudaEventDestroy(x);
  if (e != cudaSuccess) return cuda_fail(c, e, "dml_get_atoms_batch copies");
  int err = 0;
  CK(cudaMemcpyAsync(&err, ds + o_err, sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (err) return DML_E_STATE;  // sys%alist and the atom count disagree
  for (int r = 0; r < nrep; ++r) atoms[r].n = (int32_t)(off[r + 1] - off[r]);
  return 0;
}

int dml_get_atoms(dml_ctx* c, dml_atoms* a) {
  if (!c || !a) return DML_E_ARG;
  if (c->D.nrep != 1) return DML_E_ARG;
  return dml_get_atoms_replica(c, 0, a);
}

// Replica `rep`'s Verlet lists by hs%ref rank, entries as sys%alist positions
// (-1 for an atom in limbo).
int dml_get_neighbors_replica(dml_ctx* c, int32_t rep, int32_t* n_ref, int32_t* nn,
                              int32_t* list, int32_t ld) {
  if (!c || !n_ref || !nn || !list || rep < 0 || rep >= c->D.nrep) return DML_E_ARG;
  if (!c->loaded) return DML_E_STATE;
  int rc = read_scalars(c);
  if (rc) return rc;
  const Dev& d = c->D;
  cudaStream_t s = c->stream;
  const int B = c->rc[rep].base;
  const int ns = c->h_sc[rep].n_slots, nr = c->h_sc[rep].n_rank, nal = c->h_sc[rep].n_alist;
  const int mnb = c->P.mnb;
  std::vector<int> ref(nr), hnn(ns), alist(nal);
  std::vector<int8_t> st(ns);
  if (nr) CK(cudaMemcpyAsync(ref.data(), d.ref + B, sizeof(int) * nr, cudaMemcpyDeviceToHost, s));
  if (nal) CK(cudaMemcpyAsync(alist.data(), d.alist + B, sizeof(int) * nal, cudaMemcpyDeviceToHost, s));
  if (ns) {
    CK(cudaMemcpyAsync(hnn.data(), d.nn + B, sizeof(int) * ns, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(st.data(), d.state + B, ns, cudaMemcpyDeviceToHost, s));
  }
  CK(cudaStreamSynchronize(s));
  // local slot -> sys%alist position
  std::vector<int> pos_of(ns, -1);
  int q = 0;
  for (int i = 0; i < nal; ++i)
    if (alist[i] >= 0) {
      int h = alist[i] - B;
      if (h < 0 || h >= ns) return DML_E_STATE;
      pos_of[h] = q++;
    }
  std::vector<int> row(mnb);
  int k = 0;
  for (int r = 0; r < nr; ++r) {
    int h = ref[r];
    if (h < 0) continue;
    h -= B;
    if (h < 0 || h >= ns) return DML_E_STATE;
    int cnt = hnn[h];
    if (cnt > ld) return DML_E_ARG;
    if (cnt)
      CK(cudaMemcpy(row.data(), d.list + (size_t)(B + h) * mnb, sizeof(int) * cnt,
                    cudaMemcpyDeviceToHost));
    nn[k] = cnt;
    for (int e = 0; e < cnt; ++e) {
      int j = row[e] - B;
      if (j < 0 || j >= ns) return DML_E_STATE;
      list[(size_t)k * ld + e] = st[j] == ST_LIMBO ? -1 : pos_of[j];
    }
    ++k;
  }
  *n_ref = k;
  return 0;
}

int dml_get_neighbors(dml_ctx* c, int32_t* n_ref, int32_t* nn, int32_t* list, int32_t ld) {
  if (!c) return DML_E_ARG;
  if (c->D.nrep != 1) return DML_E_ARG;
  return dml_get_neighbors_replica(c, 0, n_ref, nn, list, ld);
}

}  // extern "C"
