// dml_internal.h - device data layout and kernel launchers shared by the
// C-ABI host code (dml_api.cu) and the kernels (dml_kernels.cu).
//
// Layout in HBM.  Atoms are addressed by their slot in the reference's
// `hs` ngroup index (src/Neighbor.F90:32-79); the neighbour list stores hs
// slots, so every per-atom array is indexed by hs slot:
//   pos      double4 (x, y, z, 0)            32 B, one sector per gather
//   posf     float4  (x, y, z, element bits)  16 B, the FP32 pre-filter copy
//   posf_old float4  FP32 copy of pos_old (displacement test)
//   vel, acel, force, old_cg, pos_old, ranv  double4
//   epot double, typ/skip/state int8, id int64, rank/bslot int32
// `ref` holds hs slots in hs%ref order (holes = -1 after captures); ranks
// are positions in it.  The Verlet list is row-major [slot][mnb] int32.
// Cells are a counting sort of hs%b slots into (n1+2)(n2+2)(n3+2) bins,
// each bin ordered by descending b slot (the LIFO chains of
// src/Cells.F90:299-300).
#ifndef DML_INTERNAL_H
#define DML_INTERNAL_H

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/dml.h"

namespace dml {

enum { ST_NULL = 0, ST_LIVE = 1, ST_LIMBO = 2 };

// The first statement of every kernel.  In the step graphs the edges between
// kernels are programmatic (dml_api.cu, programmatic_edges): a kernel may be
// launched before the kernel it follows has completed, and waits here until
// that kernel's writes are visible.  Without such an edge (eager launches)
// the wait returns at once.
#if defined(__CUDA_ARCH__)
#define DML_GRID_WAIT() asm volatile("griddepcontrol.wait;" ::: "memory")
#else
#define DML_GRID_WAIT() ((void)0)
#endif

constexpr int kNearCap = 32;   // near-contact entries per atom (overlap)
constexpr int kBlock = 256;
constexpr int kSlotU = 4;                 // positions per thread of the per-position kernels
constexpr int kSpan = kBlock * kSlotU;    // positions per block; replica capacities are multiples
constexpr int kCellChunk = kBlock * 4;    // cells per block of the per-cell kernels
constexpr int kCntStride = 32, kCntGlist = 0, kCntAct = 1;  // pr_cnt layout
// overlap_moveback's bookkeeping: a replica with at most this many listed
// members is handled by one block (overlap_comp_kernel), a larger one by
// grid kernels over all its listed members
constexpr int kCompBlockMax = 4096;
constexpr int kCompThreads = 512;   // overlap_comp_kernel's block
constexpr int kCntGcmcPar = 2, kCntGcmcSeq = 3;  // gcmc_run calls per path (diagnostic)

// Replicas.  A context holds one or more independent systems ("replicas",
// the batched form); a single system is a batch of one.  Replica r owns the
// positions [base, base + cap) of every per-atom array (hs slots, hs%b
// slots, hs%ref ranks, sys%alist and gcmc%alist positions), with cap a
// multiple of kSpan, so every thread block of the per-position kernels lies
// inside one replica and loads its replica's constants and state once.

// Per-replica constants (read-only during steps).
struct RepConst {
  double box[3], one_box[3], halfbox[3];
  double cell[3];
  float inv_cellf[3];       // 1 / cell in FP32 (cell-index estimates)
  float cellf[3], tess_hif; // cell and (ncells_z + 1) * cell_z in FP32 (range tests)
  float boxf[3], halfboxf[3];
  int ncells[3];
  int head_dim[3];          // ncells + 2
  int use_cells;
  int list_thread;          // list build one thread per row (sparse cells), else a warp
  int cell_off, ncell;      // this replica's cells [cell_off, cell_off + ncell), then
                            // one sentinel cell (always empty) whose start is the end
  int cch0;                 // its first chunk of kCellChunk cells (per-cell kernels)
  int base, cap, nblk;      // positions [base, base + cap), cap / kSpan blocks
  unsigned long long seed;  // Philox key of this replica
  // FP32 pre-filter bounds of this replica: the error margin of an FP32
  // coordinate difference (64 ulps of twice the largest coordinate, at least
  // 1e-3 Å) and the squared cut-offs widened or narrowed by it
  float margin;
  float rlist_lo2, rlist_hi2, rc_lo2, rc_hi2;
  float r0f_pref2[3][3];    // (r0 + margin)^2 per element pair
  // z layers of cells that gcmc_run's searches reach (bit c3, 1 <=
  // ncells[2]); gl_all: every layer (its cell sort then covers them all)
  unsigned long long gl_mask;
  unsigned long long gl_cmask;  // of those, the layers whose atoms can be within reach in z
  int gl_all;
};

// Per-replica device state (mutable).
struct Scalars {
  double zmax, z0, z1, rho, rho0, lohi;
  double zmax_frame;  // zmax before the last maxz (salida's info line)
  unsigned long long try_, depo, choques, choques3, nupd, gcmc_ins, gcmc_del;
  int n_slots;     // hs%amax (local slots in use)
  int n_b;         // hs%b%amax
  int n_rank;      // rank positions in use (members + holes)
  int n_ref;       // hs%ref%nat
  int n_atoms;     // sys%nat
  int listed;      // neighbour list built
  int rebuild;     // set by the displacement test
  int max_nn;
  int passes;      // passes of the last overlap_moveback
  int again, again2;     // overlap pass flags (pass p-1, pass p) when captures can fail
  int comp_defer;        // prob >= 1: this call's components run in overlap_pass1_kernel
  // The force scan between full scans (KParams::short_scan): the rows it
  // walks are those flagged at the replica's last full scan (an entry
  // within sl_rs) or written since; valid while every list entry's
  // displacement since then stays under sl_disp.
  float sl_disp;         // bound on any atom's displacement since the last full scan (A)
  float sl_rs;           // the flag radius of the last full scan (A)
  int sl_mode;           // this step's scan: 1 full (flags rewritten), 0 flagged rows only
  int sl_full;           // the next scan must be full (lists rebuilt, state changed by the host)
  unsigned long long sl_nfull, sl_npartial;  // steps of each mode so far
  unsigned long long dt_tests, dt_exact;     // displacement tests, those decided in FP64
  unsigned int ticket;   // last-block-done counters of this replica
  unsigned int ticket2;
  int rho_count;
  int n_new_cg;
  // structure (GCMC insertions and deletions)
  int n_alist;     // positions used in alist (members + holes)
  int n_gorder;    // positions used in gorder (members + holes)
  int n_gcmc;      // gcmc%nat
  int nlimbo;      // hs%nlimbo
  int b_nat;       // hs%b%nat
  int free_lo;     // every local hs slot below this one is in use (live or limbo)
  int bfree_lo;    // every local hs%b slot below this one holds an atom
  int halo;        // an atom sat in a halo cell at the last cell sort
  int dec;         // displacement test: 0 keep, 1 rebuild, 2 decided in FP64
  float thr;       // its FP32 candidate threshold for the FP64 top-2
  int xbeg, xcnt;  // dec 2: its spans listed for the exact pass (Dev::xspan)
  long long next_id;
};

// Context-wide device state.
struct Global {
  long long step;
  unsigned int delta2f_bits;  // FP32 upper bound of max |pos - old_cg|^2 over hs%ref (bits)
  int error;       // first dml_status raised on the device
  int err_info;
  int err_rep;
  int again;       // overlap pass produced a move-back
  int passes;      // passes of the last overlap_moveback (max over replicas)
  int n_comp;      // overlap components
  int comp_total;  // members over all components
  int n_cand;      // entries in the force candidate queue
  int any_rebuild; // some replica rebuilds its list this test_update
  unsigned int ticket_rep;  // replicas finished with the displacement test
  int n_xspan;               // spans listed for the exact displacement pass
  long long list_builds;    // rebuild kernels run (some replica rebuilt)
  int near_stale;           // near lists must be searched in the overlap phase
  int n_big;                // entries of big_cells
  int n_ftouch;             // entries of ftlist (mixed-form sums)
  int chunk_event;          // some replica added its chunk this step (bloques)
  int n_f;                  // entries of Dev::flist
};

struct EvRec {            // one interacting list entry seen from one atom
  unsigned long long key; // rank(o1) << 32 | jj : the reference's summation order
  double fx, fy, fz;      // aux*vd/dr of the entry (o1 - o2 orientation)
  double e;               // aux*0.5
  int sign;               // +1 o1 side (force += t), -1 o2 side (force -= t)
  int pad;
};

// Constants computed on the host with the reference's operation order and
// passed by value to every kernel.
struct KParams {
  double rc2;               // rc*rc (hs%rcut2)
  double rlist2;            // (rc+skin)^2
  double skin;
  double eps[3][3], r0sq[3][3], b0[3][3], c0[3][3];  // b0 = r0^6, c0 = eps*12*b0
  int pair_on[3][3];        // eps != 0 (other pairs add signed zeros only)
  // mixed form: FP32 force vectors, int64 fixed-point sums
  int mixed;
  int scan_lanes;           // lanes per list row in the force scan (1 .. 32; tuned)
  int near_lanes;           // lanes per list row in the near search (1 .. 32; tuned)
  int short_scan;           // Ermak force scan of flagged rows between full scans (no piston/chunks)
  float short_skin;         // flag radius beyond the scan's own radii (A)
  double c12[3][3];         // 12 eps / r0^2 (scalar pair force of the mixed form)
  int cand_cap;
  float rcf;                // rc (FP32, pre-filters)
  double beta_t[3];         // sqrt(kB T / m) per element (gcmc_run's Maxwell draw)
  double inv_mass[3];       // 1 / m (ermak_b of the mixed form)
  double fix_scale, fix_inv; // 2^32 per eV/Å in ui/Å, and its inverse
  double mass[3];
  // Ermak (set_ermak, dana.F90:947-971)
  double cc0, cc1, cc2, cc2h, cc1mcc2, crv1, crv2;
  double rfac[3], vfac[3];  // (skt/sqrt(m))*sdr, (skt/sqrt(m))*sdv per element
  // Brownian
  double fac_sc, fac_sei, dif_switch_z, h;
  double prob;
  double h_over_tau;
  double ztop_is_z1;        // chunks: calc_rho uses z1
  int rho_fused;            // piston: calc_rho's count taken by the step's second pbc_dispmax
  // chunk reservoir (bloques, dana.F90:716-773): chunk height, the density
  // it keeps (rhomedia, dana.F90:445) and the cell edge bound rc + skin
  double chunk_dist, rhomedia, rcut_b;
  int n_chunk;
  int integrator, reservoir;
  int mnb, ev_cap, max_passes;
  // gcmc_run (dana.F90:590-713)
  double act, beta_num;     // beta = sqrt(beta_num / mass), beta_num = kB(module) * T
  int nadj;
  // chosen form: the velocity-side constants in FP32
  float cc0f, cc1f, cc2f, cc2hf, cc1mcc2f, crv1f, crv2f;
  float rfacf[3], vfacf[3], inv_massf[3];
  float fac_scf, fac_seif, inv_hf;
};

// Chosen form: velocities and accelerations are FP32, both in the `vel`
// slot of the atom (velocity in its first 16 bytes, acceleration in its last
// 16, each a float4 (x, y, z, 0)), so ermak_a reads and ermak_b writes one
// 32-byte sector; copies and zeroing of the slot work as in the plain form.
// The Ermak velocity noise is a float4 array of its own (ranvf).
__host__ __device__ inline double4 pack_f3(float x, float y, float z) {
  double4 r = {0.0, 0.0, 0.0, 0.0};
  float f[4] = {x, y, z, 0.0f};
  unsigned char* dst = reinterpret_cast<unsigned char*>(&r);
  const unsigned char* src = reinterpret_cast<const unsigned char*>(f);
  for (int i = 0; i < 16; ++i) dst[i] = src[i];
  return r;
}
__host__ __device__ inline float4 unpack_f3(const double4& v) {
  float f[4];
  const unsigned char* src = reinterpret_cast<const unsigned char*>(&v);
  unsigned char* dst = reinterpret_cast<unsigned char*>(f);
  for (int i = 0; i < 16; ++i) dst[i] = src[i];
  return make_float4(f[0], f[1], f[2], 0.0f);
}

// gcmc_run of a replica with linked cells (the trials' searches limited to
// the 27 cells around each trial point): per-trial data found in parallel
// before the trials are decided in order.
constexpr int kGcmcMaxTrials = 256;  // trials per call on this path (nadj)
constexpr int kGcmcMaskW = kGcmcMaxTrials / 32;
constexpr int kGcmcBlk = 8;          // gcmc members within rc of a trial point
constexpr int kGcmcCand = 48;        // atoms within rc + skin of a trial point (<= 64)

struct GcmcTrialPre {
  double4 r;                 // trial point (dana.F90:643-645)
  double coin, uacc, upick;  // the trial's uniforms (dana.F90:627-686)
  unsigned long long kpick;  // upick * 2^53 (the 53-bit integer it is made of)
  double nv[3];              // Maxwell normals of an insertion (dana.F90:666-668)
  int cell;                  // linear cell of the point
  int n_blk;                 // gcmc members within rc (their gcmc%alist positions)
  int n_cand;                // atoms within rc + skin of the 27 cells, stencil order
  unsigned dup;              // bit q: stencil cell q repeats an earlier one
  int cells[27];             // the stencil cells (map order)
  int blk[kGcmcBlk];
  int cand[kGcmcCand];       // hs slots
  unsigned char cq[kGcmcCand];  // stencil index of the candidate
  unsigned char cf[kGcmcCand];  // 1: own list (rd < (rc+skin)^2), 2: append (rd <= ...)
  unsigned ckey[kGcmcCand];     // ~hs%b slot of the candidate (its order within a cell)
};

struct GcmcRepPre {
  int fast;                  // this replica's trials run on the parallel path
  int n_in, first, last, ng; // in-slab members, first/last member position, positions used
  int n_holes, n_bholes;     // free hs / hs%b slots found (the first ones, ascending)
  int holes[kGcmcMaxTrials], bholes[kGcmcMaxTrials];
};

// All device buffers of one context.
struct Dev {
  double4 *pos, *vel, *acel, *force, *old_cg, *pos_old, *ranv;
  float4* ranvf;      // chosen form: FP32 Ermak velocity noise
  float4 *posf, *posf_old;
  double* epot;
  int8_t *typ, *skip, *state, *active;
  long long* id;
  int *rank, *bslot, *ref, *b2hs;
  int *nn, *list;
  // cells
  int *cell_of, *cell_count, *cell_start, *cell_fill, *cell_atoms;
  int ncell_tot;
  // force candidate queue (rank, jj, o1 slot, o2 slot)
  int4* cand;
  // mixed form: per-atom int64 fixed-point force (x, y, z) and energy
  long long* facc;
  // mixed form: the slots whose accumulators received a pair this call,
  // one bit per slot (ftouch) and listed once each (ftlist, Global::n_ftouch)
  unsigned* ftouch;
  // chosen form: one bit per slot, set where force/epot may be nonzero (written
  // by a sum, an insertion or a load); force_ref writes the zeros of a member
  // with no pair only where the bit is set
  unsigned* fnz;
  int* ftlist;
  // hs slots whose element became F (captured) since the last capture commit
  int* flist;
  // force events
  int* ev_count;
  EvRec* ev;
  // structure: sys%alist and gcmc%alist orders (hs slots, holes = -1)
  int *alist, *apos, *gorder, *gpos;
  int8_t* in_gcmc;
  int *ins_head, *ins_next;  // atoms inserted at cell-chain heads during gcmc_run
  // overlap
  int *near_count, *near, *uf, *comp_size, *comp_id, *comp_rank, *comp_fill, *comp_members, *comp_list;
  int* act_list;      // ranks of the hs%ref members with a near contact this step, replica
                      // r's at [base, base + pr_cnt[r * kCntStride + kCntAct])
  int* rowflag;       // cap: the row takes part in the force scans between full scans
  int* sl_rows;       // cap: the flagged rows (hs slots), replica r's from its base
  int* sl_pre;        // nrep + 1: prefix of the flagged rows of the replicas scanned partially
  int* sl_nrows;      // nrep: entries of each replica's flagged-row list (not in Scalars:
                      // gcmc_run's kernels keep the scalars in shared memory and write them
                      // back, while their appends list rows)
  int* act_big_pre;   // nrep + 1: prefix of the listed members of the replicas with more
                      // than kCompBlockMax of them (0 for the others)
  int2* glist;        // gcmc_run's cell sort: (hs slot, cell) of the atoms within reach,
                      // replica r's entries at [base, base + pr_cnt[r * kCntStride + kCntGlist])
  float4* glp;        // the same entries' FP32 positions, w = hs slot (integer bits)
  float4* gsort;      // glp ordered by cell row (gcmc_pre_kernel), replica r's from base
  int* pr_cnt;        // per-replica list counters, one 128-byte line per replica (kept
                      // apart from the replica scalars that every block reads)
  // reductions
  unsigned long long* part;  // per-block partials (top-2, as double bits)
  int nblk_part;
  // The displacement test's exact pass: the spans it walks (global span
  // indices, each undecided replica's contiguous from Scalars::xbeg) and
  // their partial top-2 (2 per listed span)
  int* xspan;
  unsigned long long* xpart;
  // The step's second test_update: the FP32 top-2 of every block from the
  // first one (part1, two float bit patterns per block), and the blocks
  // where overlap_moveback moved an atom since (dirty)
  unsigned* part1;
  int* part_cnt;       // 2 per block: the reservoir-slab count of the first pass, of the current one
  int* dirty;
  // replicas
  Scalars* sc;        // [nrep] per-replica state
  Global* g;          // context-wide state
  RepConst* rc;       // [nrep] per-replica constants
  int* rep_of;        // [cap] replica of every position
  int* rank_pre;      // [nrep + 1] prefix of the replicas' n_rank (rows in use),
                      // taken at the start of each step (n_rank changes in gcmc_run)
  int* rebc_pre;      // [nrep + 1] prefix of the cell chunks of the replicas that rebuild
  int *chunk_sum, *chunk_base;  // [n_cch] cell counts per chunk, first cell_atoms place
  int* reb_pre;       // [nrep + 1] the same prefix over the replicas whose list the
                      // last displacement test rebuilds (0 rows for the others)
  int* big_cells;     // cells too large for the per-thread sort of cell_order
  int* cch_rep;       // [n_cch] replica of every chunk of kCellChunk cells
  int n_cch;
  // gcmc_run on the parallel path (allocated with the GCMC reservoir)
  GcmcTrialPre* gpre;  // [nrep][kGcmcMaxTrials]
  unsigned* gpm;       // [nrep][kGcmcMaxTrials][kGcmcMaskW] earlier trial points within rc
  GcmcRepPre* grp;     // [nrep]
  unsigned *gw_mem, *gw_slab;  // [cap / 32] membership / in-slab bits of gcmc%alist positions
  // chunk reservoir: every replica's template atoms (positions and old
  // positions, [nrep][n_chunk]) and their elements ([n_chunk])
  double4 *chk_pos, *chk_pold;
  int8_t* chk_typ;
  int nrep;
  int cap;            // positions over all replicas (sum of the replica caps)
  int max_rep_cap;    // largest replica capacity
  int gcmc_rows;      // most cell rows (z layer, y row) of a replica with cells
  int any_cells, any_verlet;  // some replica uses linked cells / the all-pairs build
  int any_list_thread, any_list_warp;  // the mappings of the cell list builds in use
};

// Compact per-atom input of dml_set_atoms_batch on the device: the replicas'
// atoms concatenated (replica r's at [off[r], off[r + 1])), absent optional
// arrays NULL.  rk / gk: the atom's place in hs%ref / gcmc%alist, or -1.
struct LoadIn {
  const double *pos, *vel, *acel, *force, *pos_old, *old_cg, *epot;
  const int *z, *rk, *gk, *off;
  const int8_t* skip;
  const long long* id;
  int n_tot;
};

// ---- kernel launchers (dml_kernels.cu); each returns the kernels it queued ----
int k_load_atoms(const Dev& d, const KParams& p, const LoadIn& in, cudaStream_t s);
// Output of dml_get_atoms_batch on the device: per member a packed array
// over all replicas (replica r's atoms from off[r]); NULL members are skipped.
struct PackOut {
  double *pos, *vel, *acel, *force, *pos_old, *old_cg, *epot;
  int* z;
  int8_t *skip, *in_ref, *in_gcmc;
  long long* id;
  const long long* off;  // [nrep + 1]
  int* err;              // set when a replica's live count differs from off
};
int k_pack_atoms(const Dev& d, const KParams& p, const PackOut& o, cudaStream_t s);
int k_salida(const Dev& d, const KParams& p, double kb, dml_observables* out, cudaStream_t s);
int k_check_conversions(const double* x, float* f32, double* back, long long n, cudaStream_t s);
int k_check_normals(const unsigned* w, float* out, long long n_pairs, int fast,
                    cudaStream_t s);
int k_check_pick(const unsigned long long* k, const int* n, int* m, long long count, cudaStream_t s);
int k_step_begin(const Dev& d, int near_stale, cudaStream_t s);
int k_rank_prefix(const Dev& d, cudaStream_t s);
int k_ermak_a(const Dev& d, const KParams& p, int n_rank, cudaStream_t s);
int k_brownian(const Dev& d, const KParams& p, int n_rank, cudaStream_t s);
int k_force_pairs(const Dev& d, const KParams& p, int n_rank, bool near, cudaStream_t s);
int k_force_scan(const Dev& d, const KParams& p, int n_rank, bool near, cudaStream_t s);
int k_reset_candidates(const Dev& d, cudaStream_t s);
int k_scan_invalidate(const Dev& d, cudaStream_t s);
int k_force_sum(const Dev& d, const KParams& p, int n_slots, bool fuse_ermak_b, cudaStream_t s);
int k_ermak_b(const Dev& d, const KParams& p, int n_rank, cudaStream_t s);
// second: the step's test_update after overlap_moveback, which recomputes
// only the blocks where an atom moved since the first one.
int k_test_update(const Dev& d, const KParams& p, int n_slots, int n_b, int n_rank,
                  cudaStream_t s, bool second = false);
int k_pbc_dispmax_cond(const Dev& d, const KParams& p, int n_slots,
                       cudaGraphConditionalHandle h, cudaStream_t s, bool second = false);
int k_rebuild(const Dev& d, const KParams& p, int n_slots, int n_b, int n_rank, cudaStream_t s);
// overlap_moveback: standalone (its own delta and near search) or as the
// second half of a fused step whose first half ran k_overlap_prepare.
int k_overlap_prepare(const Dev& d, const KParams& p, int n_slots, cudaStream_t s);
// detect: 0 no near search (done elsewhere), 1 only if the near lists are
// stale, 2 always.
int k_overlap(const Dev& d, const KParams& p, int n_rank, int n_slots, bool standalone,
              int detect, cudaStream_t s);
int k_overlap_detect(const Dev& d, const KParams& p, int n_rank, int mode, cudaStream_t s);
int k_capture_commit(const Dev& d, const KParams& p, int n_rank, cudaStream_t s);
int k_calc_rho(const Dev& d, const KParams& p, int n_slots, cudaStream_t s);
// bloques: the chunk event of every replica (sets Global::chunk_event); with
// a conditional handle the kernel after it opens the rebuild subgraph.
int k_bloques(const Dev& d, const KParams& p, cudaStream_t s);
int k_chunk_cond(const Dev& d, cudaGraphConditionalHandle h, cudaStream_t s);
int k_piston(const Dev& d, const KParams& p, int n_slots, cudaStream_t s);
int k_flush(void* buf, size_t bytes, cudaStream_t s);
int k_gcmc(const Dev& d, const KParams& p, int cap, cudaStream_t s);
int k_gcmc_cells(const Dev& d, const KParams& p, int cap, cudaStream_t s);
int k_gcmc_trials(const Dev& d, const KParams& p, cudaStream_t s);
int k_pbc_dispmax(const Dev& d, const KParams& p, int n_slots, cudaStream_t s,
                  bool second = false);

}  // namespace dml

#endif
