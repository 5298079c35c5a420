/*
 * dml.h - C ABI of the GB300 (sm_103a) implementation of din-mol-Li's
 * per-step hot path.
 *
 * The reference exposes no library interface: its hot path is a set of
 * internal procedures of `program dana` (src/dana.F90) that read
 * host-associated globals and walk linked lists of `atom` objects.  Each entry
 * point below replaces one of those procedures, so a driver written like
 * dana.F90 calls `dml_ermak_a` where dana.F90 calls `ermak_a`, and so on.
 * The replaced procedure is cited beside each declaration.
 *
 * Conventions
 *  - Every call returns 0 on success or a positive `dml_status` code; the
 *    codes mirror the reference's `werr` / `stop` sites.  `dml_strerror`
 *    gives the message.  A failed call leaves the context usable only for
 *    `dml_get_*`, `dml_last_error` and `dml_destroy`.
 *  - The context owns all device memory.  Host arrays passed in are read
 *    during the call only.
 *  - Atom arrays are given in the order of the reference's `sys%alist`
 *    (attachment order).  Membership of `hs%ref` is a flag per atom; the
 *    iteration order of `hs%ref` is `sys%alist` order restricted to members,
 *    exactly as in the reference (both lists only ever append and remove).
 *  - A context is used from one host thread.  All work is queued on the
 *    context's own CUDA stream; calls return after the stream is idle.
 *  - Coordinates are Å, masses amu, time ps, energies ui = amu Å^2 ps^-2.
 */
#ifndef DML_H
#define DML_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DML_ABI_VERSION 1

typedef enum dml_status {
  DML_OK = 0,
  DML_E_ARG = 1,                 /* invalid argument */
  DML_E_CUDA = 2,                /* CUDA runtime error (message via dml_last_error) */
  DML_E_NOMEM = 3,               /* device or host allocation failed */
  DML_E_OUT_OF_TESSELLATION = 4, /* src/Cells.F90:293-294 "Particle out of tessellation" */
  DML_E_UNSORT = 5,              /* src/Cells.F90:350 "Unsort cgroup particle fail" */
  DML_E_INDEX = 6,               /* src/Groups.F90:1088 "Index inconsistency" */
  DML_E_NO_PARTICLES = 7,        /* src/dana.F90:624 "No more particles" */
  DML_E_CHOSEN_MISSING = 8,      /* src/dana.F90:701 "Chosen particle does not exists" */
  DML_E_RESERVOIR = 9,           /* src/dana.F90:423 "Unknown reservoir type" */
  DML_E_DENDRITE = 10,           /* src/dana.F90:905-908 deposit above z0 ("supero z0", stop) */
  DML_E_RSA = 11,                /* src/dana.F90:386-389 placement tries exhausted */
  DML_E_OVERLAP_PASSES = 12,     /* overlap_moveback recursion exceeded the pass cap */
  DML_E_NEIGH_OVERFLOW = 13,     /* more than mnb neighbours (src/Neighbor.F90:44) */
  DML_E_EVENT_OVERFLOW = 14,     /* per-atom interaction bucket overflow (force path) */
  DML_E_FIXEDPOINT_OVERFLOW = 15,/* mixed form: force beyond the int64 fixed-point range */
  DML_E_CAPACITY = 16,           /* atom capacity exceeded */
  DML_E_UNSUPPORTED = 17,        /* option not implemented on the device */
  DML_E_NEAR_OVERFLOW = 18,      /* overlap near-contact bucket overflow */
  DML_E_STATE = 19               /* call out of order (e.g. step before set_atoms) */
} dml_status;

enum { DML_INTEGRATOR_BROWNIAN = 0, DML_INTEGRATOR_ERMAK = 1 };
enum { DML_RESERVOIR_NONE = 0, DML_RESERVOIR_PISTON = 1, DML_RESERVOIR_CHUNKS = 2, DML_RESERVOIR_GCMC = 3 };
enum { DML_PRECISION_FP64 = 0, DML_PRECISION_MIXED = 1 };
enum { DML_Z_LI = 1, DML_Z_CG = 2, DML_Z_F = 3 };

/* Run parameters.  The reference reads them from entrada.ini / movedor.ini
 * (src/dana.F90:309-327, 399-427) or hard-codes them (src/dana.F90:12-25,
 * 81-100, 113).  dml_params_default fills the hard-coded values. */
typedef struct dml_params {
  double box[3];          /* tbox diagonal: xi, yi, box height (src/dana.F90:342-346) */
  double z0;              /* reservoir bottom */
  double zmax;            /* reservoir top (moves with the piston) */
  double z1;              /* chunk-reservoir sensor top (chunks only) */
  double h;               /* time step [ps] */
  double gamma;           /* friction [1/ps] (src/dana.F90:15) */
  double temp;            /* temperature [K] (src/dana.F90:17) */
  double kb_driver;       /* kB [ui/K] of program dana, used by set_ermak (src/dana.F90:22-24) */
  double kb_module;       /* kB [ui/K] of gems_constants, used by gcmc_run (src/Constants.F90:165-167) */
  double eps[3][3];       /* pair epsilon [ui], index [z-1][z-1] (src/dana.F90:86-100) */
  double r0[3][3];        /* pair r0 [Å] */
  double mass[3];         /* masses of Li, CG, F (src/dana.F90:82-84) */
  double rc;              /* hard-core radius = list cut radius (src/dana.F90:113) */
  double skin;            /* nb_dcut, Verlet shell (src/Neighbor.F90:109) */
  double prob;            /* capture probability */
  double dif_sc;          /* Brownian diffusion above dif_switch_z */
  double dif_sei;         /* Brownian diffusion at or below dif_switch_z */
  double dif_switch_z;    /* 80 Å (src/dana.F90:817) */
  double tau;             /* piston relaxation time (src/dana.F90:12) */
  double act;             /* GCMC activity */
  int32_t nadj;           /* GCMC trials per step */
  int32_t integrator;     /* DML_INTEGRATOR_* */
  int32_t reservoir;      /* DML_RESERVOIR_* */
  int32_t precision;      /* DML_PRECISION_* */
  int32_t mnb;            /* max neighbours per atom (reference: 10000) */
  int32_t capacity;       /* max atoms the context can hold (0: 2 x initial count) */
  int32_t max_passes;     /* overlap_moveback pass cap (0: 64) */
  int32_t event_cap;      /* interacting entries per atom per step, force path (0: 64) */
  uint64_t seed;          /* Philox key */
} dml_params;

/* Atom state in sys%alist order.  Arrays are [n] or [n][3] (x,y,z innermost).
 * Output pointers that are NULL are skipped by dml_get_atoms. */
typedef struct dml_atoms {
  int32_t n;
  double* pos;      /* [n][3] */
  double* vel;      /* [n][3] */
  double* acel;     /* [n][3] */
  double* force;    /* [n][3] */
  double* pos_old;  /* [n][3] position at the last neighbour-list build */
  double* old_cg;   /* [n][3] position at the start of the step */
  double* epot;     /* [n] */
  int32_t* z;       /* DML_Z_* */
  int8_t* skip;     /* overlap_moveback flag */
  int8_t* in_ref;   /* member of hs%ref (mobile) */
  int8_t* in_gcmc;  /* member of the gcmc group */
  int64_t* id;      /* persistent atom id (Philox key) */
} dml_atoms;

/* Run counters (src/dana.F90:30-33, 50; src/Neighbor.F90:110-111). */
typedef struct dml_counters {
  int64_t try_;       /* capture attempts since the last reset (try) */
  int64_t depo;       /* captures since the last reset (depo) */
  int64_t choques;    /* ion-ion move-backs */
  int64_t choques3;   /* unresolved piston overlaps */
  int64_t nupd;       /* neighbour-list rebuilds (nupd_vlist) */
  int64_t step;       /* steps done */
  int64_t gcmc_ins;   /* accepted insertions */
  int64_t gcmc_del;   /* accepted deletions */
  int32_t n_atoms;    /* sys%nat */
  int32_t n_ref;      /* hs%ref%nat */
  int32_t max_nn;     /* largest neighbour count of the last build */
  int32_t passes;     /* overlap passes in the last overlap_moveback */
  double zmax;        /* current zmax */
  double z0;          /* current z0 */
  double rho;         /* last calc_rho */
  double rho0;        /* initial rho */
  int64_t list_builds; /* test_updates that rebuilt some replica's list (one
                          launch of the rebuild kernels each) */
} dml_counters;

typedef struct dml_ctx dml_ctx;

/* Fills the reference's hard-coded constants (src/dana.F90:12-25,81-100,113;
 * src/Constants.F90:165-167) and the tests/ermak run values. */
void dml_params_default(dml_params* p);

/* Creates a context on the current CUDA device.  Allocates device memory
 * for `capacity` atoms and their neighbour lists. */
int dml_create(const dml_params* p, dml_ctx** out);

/* Loads atoms (replaces config_inic, src/dana.F90:430-517, and the gcmc
 * attach loop :130-137).  Marks the neighbour list as not built. */
int dml_set_atoms(dml_ctx* c, const dml_atoms* a);

/* Independent replicas in one context (no counterpart in the reference,
 * which runs one system per process; each replica is one `dana` run).
 * Every replica has its own box, electrode plane z0, piston zmax, chunk
 * plane z1 and random seed; all share the remaining dml_params (potential,
 * integrator, reservoir, capacity per replica).  Every kernel of a step
 * covers all replicas in one launch: a replica owns a block-aligned range
 * of atom slots and its own cells, lists and counters, and the results of
 * each replica are bit-identical to a one-replica context with the same
 * replica values (the Philox key carries the replica's seed).
 * dml_create is dml_create_batch with one replica taken from p. */
typedef struct dml_replica {
  double box[3];
  double z0, zmax, z1;
  uint64_t seed;
} dml_replica;

int dml_create_batch(const dml_params* p, int32_t n_rep, const dml_replica* reps,
                     dml_ctx** out);

/* Loads atoms[r] into replica r for r in [0, n_rep).  dml_set_atoms is the
 * one-replica form and fails with DML_E_ARG on a context of several. */
int dml_set_atoms_batch(dml_ctx* c, const dml_atoms* atoms);

/* Replica count of a context, or -status. */
int dml_num_replicas(dml_ctx* c);

/* set_ermak (src/dana.F90:947-971) + test_update (:140) + fuerza (:142) +
 * calc_rho (:145, sets rho0): the start-up sequence before the step loop. */
int dml_setup(dml_ctx* c);

/* test_update (src/Neighbor.F90:668-713): do_pbc, cell sort and the
 * displacement test; rebuilds the Verlet list when needed.  *rebuilt is set
 * to 1 when the list was rebuilt (may be NULL). */
int dml_test_update(dml_ctx* c, int32_t* rebuilt);

/* fuerza (src/dana.F90:1055-1139): pair forces and energies over the list. */
int dml_force(dml_ctx* c);

/* ermak_a (src/dana.F90:974-1028) with atom_pbc (:1187-1250) for step `step`. */
int dml_ermak_a(dml_ctx* c, int64_t step);

/* ermak_b (src/dana.F90:1031-1052). */
int dml_ermak_b(dml_ctx* c);

/* cbrownian_hs (src/dana.F90:798-846) with atom_pbc for step `step`. */
int dml_brownian(dml_ctx* c, int64_t step);

/* overlap_moveback (src/dana.F90:849-943) for step `step`. */
int dml_overlap_moveback(dml_ctx* c, int64_t step);

/* Capture commit loop (src/dana.F90:226-236): F -> CG, detach from hs%ref
 * and gcmc.  *n_new may be NULL. */
int dml_capture_commit(dml_ctx* c, int32_t* n_new);

/* gcmc_run (src/dana.F90:590-713) for step `step`. */
int dml_gcmc(dml_ctx* c, int64_t step);

/* calc_rho (src/dana.F90:521-549).  *rho may be NULL. */
int dml_calc_rho(dml_ctx* c, double* rho);

/* maxz (src/dana.F90:776-794): piston compression using the last rho. */
int dml_piston(dml_ctx* c);

/* Chunk reservoir (reservoir DML_RESERVOIR_CHUNKS).  dml_set_chunk replaces
 * config_chunk (src/dana.F90:552-587): the n template atoms as chunk.xyz
 * gives them (pos [n][3], elements z [n]), the same for every replica, and
 * the chunk height dist (entrada.ini's dist plus rc, as config_inic makes it,
 * :437-441; z0, z1 and zmax come in dml_params / dml_replica as config_inic
 * leaves them).  It must come before dml_set_atoms_batch: the template is
 * raised by each replica's zmax there and takes the ids after the
 * replica's atoms, and each replica's cells are sized for the tallest box
 * its capacity allows ((capacity - atoms) / n chunks; default capacity:
 * room for 16 chunks).  dml_bloques replaces bloques (:716-773) with the
 * test_update it ends with; dml_step runs it after calc_rho, as the
 * reference's step does (:247). */
int dml_set_chunk(dml_ctx* c, int32_t n, const double* pos, const int32_t* z, double dist);
int dml_bloques(dml_ctx* c);

/* One or more iterations of the step loop body (src/dana.F90:173-265,
 * without the output and timer lines, with the piston's maxz and the chunk
 * reservoir's bloques), starting at step counter+1.  The steps are queued
 * as CUDA graphs (see dml_set_graph_steps) and replayed. */
int dml_step(dml_ctx* c, int64_t nsteps);

/* Queues nsteps like dml_step and returns without waiting. dml_sync waits. */
int dml_step_async(dml_ctx* c, int64_t nsteps);
int dml_sync(dml_ctx* c);

/* Steps per graph launch (no counterpart in the reference): dml_step and
 * dml_step_async queue runs of k steps as one CUDA graph (each step with its
 * own conditional rebuild nodes, built at the first run of k or more steps)
 * and the rest one step per launch.  Default 100; 1 launches one graph per
 * step.  The results do not depend on k. */
int dml_set_graph_steps(dml_ctx* c, int32_t k);

/* Benchmark support: nsteps steps queued as dml_step queues them (graphs of
 * graph_steps steps), bracketed by one pair of CUDA events on the context
 * stream; *ms is their device time.  No L2 flush. */
int dml_time_run(dml_ctx* c, int64_t nsteps, double* ms);

/* Benchmark support.  dml_time_steps queues nsteps steps like dml_step,
 * each bracketed by CUDA events on the context stream; with flush_l2 a
 * 256 MiB buffer is overwritten between steps, outside the events.  *ms is
 * the sum of the per-step device times.  dml_profile_steps runs nsteps steps
 * without the graph but with the graph's kernels (the rebuild condition of
 * each test_update is read on the host, and the idle time of that read is
 * not counted), recording an event at every phase boundary, and adds the
 * device time of phase k (DML_PHASE_*) to phase_ms[k].
 * dml_launches_per_step returns the kernels a step launches when the list is
 * not rebuilt (or -status); *per_rebuild (may be NULL) receives the kernels
 * each list rebuild adds (the rebuild is a conditional graph node). */
enum {
  DML_PHASE_INTEGRATE = 0,   /* ermak_a or cbrownian_hs (+ atom_pbc) */
  DML_PHASE_FORCE_PAIRS = 1, /* fuerza: list scan, interacting entries */
  DML_PHASE_FORCE_SUM = 2,   /* fuerza: ordered sums + ermak_b */
  DML_PHASE_TEST_UPDATE1 = 3,/* test_update after the move (+ rebuild) */
  DML_PHASE_OVERLAP = 4,     /* overlap_moveback */
  DML_PHASE_TEST_UPDATE2 = 5,/* test_update after the overlaps */
  DML_PHASE_COMMIT = 6,      /* F -> CG commit */
  DML_PHASE_GCMC_CELLS = 7,  /* gcmc_run: cell sort of the current positions */
  DML_PHASE_GCMC = 8,        /* gcmc_run: the trials (empty without GCMC) */
  DML_PHASE_RHO_PISTON = 9,  /* calc_rho + maxz */
  DML_NPHASE = 10
};
int dml_time_steps(dml_ctx* c, int64_t nsteps, int32_t flush_l2, double* ms);
int dml_profile_steps(dml_ctx* c, int64_t nsteps, int32_t flush_l2, double* phase_ms,
                      int32_t nphase);
int dml_launches_per_step(dml_ctx* c, int32_t* per_rebuild);

/* No counterpart in the reference.  The plain FP64 pair force and energy of
 * dml_force, computed over device arrays the caller owns, allocating
 * nothing.  For callers that cannot allocate device memory: a host whose
 * device memory belongs to another allocator or runtime (where a cudaMalloc
 * of this library would fail or fight that allocator), and a time-stepping
 * loop that must not call cudaMalloc or cudaFree, which stall the host.
 * Scratch lives in one static device array, held by every GPU that loads the
 * library until exit, sized for at most 16384 atoms and 32 interacting list
 * entries per atom: more atoms return DML_E_CAPACITY before any launch, more
 * entries DML_E_EVENT_OVERFLOW.
 * Inputs: pos [n][3], z [n] (DML_Z_*), the mobile atoms ref [n_ref] (atom
 * indices, in the order their forces are summed) and their neighbour lists
 * nn [n_ref], list [n_ref][ld] (atom indices, -1 for an empty entry).
 * Outputs: force [n][3] and epot [n]; the mobile atoms' values are zeroed,
 * then summed, the other atoms' values are added to.  On a nonzero return
 * force and epot are left as passed.  Results equal dml_force's bit for bit.
 * The first call on a device takes the array's address
 * (cudaGetSymbolAddress) and keeps it: make it before any stream capture,
 * and do not call after cudaDeviceReset.  Calls share the array: calls that
 * overlap on the GPU race.  The call queues on `stream` (a cudaStream_t,
 * NULL = default), reads its status back and returns when the stream is
 * idle. */
int dml_force_noalloc(const dml_params* p, int32_t n_atoms, const double* pos, const int32_t* z,
                      int32_t n_ref, const int32_t* ref, const int32_t* nn, const int32_t* list,
                      int32_t ld, double* force, double* epot, void* stream);

/* Copies atom state to host arrays (sys%alist order).  a->n must be the
 * array capacity on entry; it is set to the atom count on return. */
int dml_get_atoms(dml_ctx* c, dml_atoms* a);

/* Neighbour lists of hs%ref members in hs%ref order: nn[k] entries for the
 * k-th member, written to list[k*ld ...] as sys%alist positions (0-based).
 * Limbo entries are written as -1.  n_ref is set to the member count. */
int dml_get_neighbors(dml_ctx* c, int32_t* n_ref, int32_t* nn, int32_t* list, int32_t ld);

/* Counters of one replica.  dml_get_counters sums the event counters and
 * atom counts over replicas and reports replica 0's zmax, z0, rho, rho0
 * (max_nn and passes as maxima). */
int dml_get_counters(dml_ctx* c, dml_counters* out);

/* Autotuner result (no counterpart in the reference): the lanes per list
 * row (1, 2, 4, 8, 16 or 32) chosen, when the step graph was built, for the
 * step's per-row scan (the force scan with the Ermak integrator, the
 * near-contact search of overlap_moveback with the Brownian one), and the
 * measured time of each mapping in microseconds (scan_us[6], in that order,
 * zero before tuning).  Either pointer may be NULL. */
int dml_get_tuning(dml_ctx* c, int32_t* scan_lanes, float* scan_us);

/* Cell size of the chosen form (no counterpart in the reference, whose
 * cells are int(box / (rc + skin)) per axis; DML_PRECISION_MIXED only, not
 * with the chunk reservoir, after dml_set_atoms).  dml_set_cell_factor takes
 * cells with an edge bound of factor * (rc + skin), factor in [1, 2] (never
 * fewer than 3 cells along an axis that had 3): the lists hold the same
 * atoms in another order, which the fixed-point force sums do not see, and
 * every list is rebuilt at the next test_update.  dml_tune_cells times
 * `steps` steps with each factor 1.0, 1.1, .. 1.5 (after its rebuild step)
 * and keeps the fastest, *best (may be NULL); the run advances by
 * 6 * (steps + 1) + 1 steps.  dml_get_cell_tuning reports the factor in use
 * and the microseconds per step of each factor tried (us[6], zero if not
 * tuned).  Either pointer may be NULL. */
int dml_set_cell_factor(dml_ctx* c, double factor);
int dml_tune_cells(dml_ctx* c, int32_t steps, double* best);
int dml_get_cell_tuning(dml_ctx* c, double* factor, float* us);
int dml_get_counters_replica(dml_ctx* c, int32_t rep, dml_counters* out);

/* Diagnostic (no counterpart in the reference): how many gcmc_run calls of
 * replica `rep` ran on the parallel path (trials searched at once, decided
 * in order by one warp) and how many on the sequential one (a replica
 * without cells, an atom in a halo cell, or a search beyond the parallel
 * path's bounds).  Either pointer may be NULL. */
int dml_get_gcmc_paths(dml_ctx* c, int32_t rep, int64_t* parallel, int64_t* sequential);

/* Diagnostic (no counterpart in the reference): how many steps of replica
 * `rep` ran the force scan over all rows (a full scan, which also flags the
 * rows with an entry near enough to matter until atoms have moved by the
 * flag margin) and how many over the flagged rows only.  The second count
 * stays 0 unless the scan runs one lane per row with the Ermak integrator and
 * a GCMC or fixed reservoir.  Either pointer may be NULL. */
int dml_get_scan_counts(dml_ctx* c, int32_t rep, int64_t* full, int64_t* partial);

/* Diagnostic (no counterpart in the reference): how many displacement tests
 * (test_update's inq_dispmax, src/Neighbor.F90:635-666) replica `rep` ran
 * and how many of them the FP32 top-2 left within its error margin of the
 * skin, so that the exact FP64 pass decided.  Either pointer may be NULL. */
int dml_get_test_counts(dml_ctx* c, int32_t rep, int64_t* tests, int64_t* exact);

/* Lanes per neighbour-list row of the force scan (1, 2, 4, 8, 16 or 32;
 * with the Brownian integrator, which has no force scan, of overlap_moveback's
 * near-contact search), or 0 to let the autotuner choose when the step graph
 * is next built (the default).  The step graph is built again at the next
 * step.  Returns 0 or DML_E_ARG. */
int dml_set_scan_lanes(dml_ctx* c, int32_t lanes);

/* One replica's atoms and neighbour lists (same layout as dml_get_atoms and
 * dml_get_neighbors, which take a one-replica context). */
int dml_get_atoms_replica(dml_ctx* c, int32_t rep, dml_atoms* a);

/* Every replica's atoms at once: atoms[r] as for dml_get_atoms_replica (n
 * the capacity on entry, the count on return; NULL members are not
 * copied).  The members requested must be the same for every replica.  The
 * fields are packed on the device in sys%alist order and copied to the
 * caller's arrays, one copy per replica and member. */
int dml_get_atoms_batch(dml_ctx* c, dml_atoms* atoms);

/* The atom count of every replica (out[n_rep]), from one read of the
 * device state: the capacities dml_get_atoms_batch needs. */
int dml_get_atom_counts(dml_ctx* c, int32_t* out);
int dml_get_neighbors_replica(dml_ctx* c, int32_t rep, int32_t* n_ref, int32_t* nn,
                              int32_t* list, int32_t ld);

/* Resets try and depo (salida, src/dana.F90:1171-1174). */
int dml_reset_counters(dml_ctx* c);

/* What salida (src/dana.F90:1143-1183) writes every nwr steps for one
 * replica: units 12 to 16 and the info line of unit 11.  The frame itself
 * (unit 11's elements and positions) is dml_get_atoms_batch with z and pos. */
typedef struct dml_observables {
  int64_t step;      /* steps done */
  double energia;    /* sum of epot over sys%alist, in list order (unit 12) */
  double temp;       /* kion (src/dana.F90:1342-1376): the sum over the
                        non-CG atoms, in list order, of m (v.v), divided by
                        j * 3 * kB_ui, j their count (unit 13) */
  double rho;        /* the last calc_rho (unit 14) */
  double zmax;       /* zmax before the last maxz: the value on salida's
                        info line, which maxz follows in the step */
  int64_t try_;      /* capture attempts since the last salida (unit 15) */
  int64_t depo;      /* captures since the last salida (unit 16) */
  int32_t n_atoms;   /* sys%nat */
  int32_t n_mobile;  /* j of kion */
} dml_observables;

/* salida for every replica: out[n_rep] from one device pass over the
 * replicas' atoms, after which try and depo are zero, as salida leaves them.
 * The sums add one term at a time in sys%alist order, as the reference's
 * loops do, so they equal those loops bit for bit. */
int dml_salida(dml_ctx* c, dml_observables* out);

/* Initial configurations (replace pos_inic, src/dana.F90:330-396, which
 * cannot load an electrode).  dml_gen_bcc_slab writes, on the host, the
 * 2*nx*ny*nz atoms of a bcc lattice with constant a (corner then body-centre
 * atom per cell, x fastest) and returns the count, or -status.
 * dml_gen_ions_batch places the ions of n_sys systems on the GPU, one thread
 * block per system: system s gets specs[s].n ions in [0,box_x) x [0,box_y) x
 * [zlo,zhi) by random sequential addition, ion i keeping the first of its
 * tries whose minimum-image distance (x, y periodic) to every earlier ion is
 * at least dmin, or failing after 10 000 tries (the rule of
 * dana.F90:361-389).  The k-th try of ion i is the keyed Philox draw
 * (seed, k, i).  The result is bit-identical to placing the ions one by
 * one.  Outputs are host arrays: pos_out [sum n][3] (system s after the
 * earlier systems' ions), status [n_sys] (0 or DML_E_RSA; may be NULL).
 * Returns 0, the first nonzero system status, or DML_E_ARG / DML_E_NOMEM /
 * DML_E_CUDA / DML_E_CAPACITY (more than 2^28 grid cells).  dml_gen_ions is
 * the one-system form; it returns 0 or -status. */
typedef struct dml_ion_spec {
  uint64_t seed;
  int32_t n;
  int32_t pad;
  double box_x, box_y, zlo, zhi, dmin;
} dml_ion_spec;

int dml_gen_bcc_slab(int32_t nx, int32_t ny, int32_t nz, double a, double* pos_out, int32_t cap);
int dml_gen_ions_batch(int32_t n_sys, const dml_ion_spec* specs, double* pos_out,
                       int32_t* status);
int dml_gen_ions(uint64_t seed, int32_t n, double box_x, double box_y, double zlo, double zhi,
                 double dmin, double* pos_out);

/* Diagnostic (no counterpart in the reference): runs the device's
 * binary64 -> binary32 conversion (round to nearest, ties to even) that
 * makes the FP32 position copies, and the exact binary32 -> binary64
 * conversion that the integrators apply to FP32 increments, over n values
 * on the default stream: f32[i] = RN32(x[i]), back[i] = f32[i] as a double.
 * Host arrays; returns 0 or DML_E_CUDA. */
int dml_check_conversions(const double* x, int64_t n, float* f32, double* back);

/* Diagnostic (no counterpart in the reference): the device's Box-Muller pair
 * of the keyed streams, out[2i], out[2i+1] = the two normals made from the
 * 32-bit words words[2i], words[2i+1].  precision DML_PRECISION_FP64: the
 * pair of the plain form and of gcmc_run (include/dml_rng.h,
 * dml_normal_pair32f, bit-identical to the host build; its integer-to-float
 * steps are integer operations on the device).  DML_PRECISION_MIXED: the
 * chosen form's integrators' pair (approximate hardware log2, sin, cos).
 * Host arrays; returns 0, DML_E_ARG or DML_E_CUDA. */
int dml_check_normals(const uint32_t* words, int64_t n_pairs, int32_t precision, float* out);

/* Diagnostic (no counterpart in the reference): the device's deletion pick
 * of gcmc_run, m[i] = int(upick * n[i]) + 1 capped at n[i] with upick =
 * k[i] * 2^-53 (k[i] < 2^53), computed in integer arithmetic as the binary64
 * product rounds (src/dana.F90:686-690).  Host arrays; returns 0 or
 * DML_E_CUDA. */
int dml_check_pick(const uint64_t* k, const int32_t* n, int64_t count, int32_t* m);

const char* dml_strerror(int code);

/* Text of the last CUDA or argument error of this context. */
const char* dml_last_error(dml_ctx* c);

void dml_destroy(dml_ctx* c);

#ifdef __cplusplus
}
#endif

#endif /* DML_H */
