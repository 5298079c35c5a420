#!/usr/bin/env python3
"""Benchmark of din-mol-Li's per-step hot path on GB300.

A step is one iteration of the reference's loop body (src/dana.F90:173-265):
ermak_a, fuerza, ermak_b, test_update, overlap_moveback, test_update, capture
commit, gcmc_run, calc_rho (and maxz with the piston), all on the device.

Workloads (seeded synthetic systems; the reference measures no dataset):

  c5 (default)  config 5: a batch of independent replicas, each a 40 x 40 x
                2-cell bcc Li electrode (6400 atoms, 140.4 Å square) under
                20 000 Li+ in a 300 Å box, GCMC reservoir slab z in [200, 300]
                with 128 trials per step, Ermak, dt = 1 fs, skin 2 Å (the
                neighbour shell of the reference's GCMC run).  Timed
                in the chosen form (mixed precision, all replicas in every
                launch); the same batch in plain FP64 and a sample of replicas
                run one per context in plain FP64 are timed beside it.
  c2            config 2: one 351 x 351 x 320 Å system, 80 000 electrode atoms
                and 200 000 Li+, piston reservoir, Ermak, plain FP64 (the form
                bit-exact to the oracle).
  c4            config 4: 1024 replicas of uneven size (L x L x 2-cell
                electrode, L in 5..40 cells, 50..20 000 ions, 1 M height),
                Brownian, chosen form, all replicas in every launch.
  c3            config 3, an accuracy study rather than a bench line: config
                2's system in the chosen form against the plain FP64 form,
                force and energy errors at steps 0, K/10 and K (default K =
                10 000) and deposition counts over --seeds seeds.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--workload c5|c2|c3|c4] [--replicas R] [--form chosen|plain]

Prints one JSON line.  `value` = mobile-ion steps per second over all ranks
(device time with CUDA events, inputs resident, L2 flushed between steps);
`value_including_electrode` counts every atom, frozen electrode included.
`e2e` = the same metric through the C ABI with host arrays: upload, setup, K
steps with, every 100 steps (the reference's output cadence), what salida
writes for every replica: the frame (positions, elements) and the observables
of dml_salida (energy, temperature, rho, try, depo); wall clock.
`--impl reference` times the CPU restatement of the reference (oracle/) on
this host, one replica per host thread; rank 0 only.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "din-mol-li_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "particle-steps/s on 1 GB300: mixed+batched vs plain FP64 at force err \u22641e-6"
UNIT = "particle-steps/s"
NWR = 100  # output cadence of the reference's tests (entrada.ini nwr)

# The kernel that dominates each phase of a step, and its algorithmic bytes
# per unit.  Units: "ion" = mobile ion (hs%ref member), "slot" = atom of hs%b
# (electrode included), "trial" = GCMC trial.  Per ion: integrate reads pos,
# vel, acel and writes pos, old_cg (120 B); force_sum (+ ermak_b) reads the
# force accumulators, vel, acel, element and writes vel, acel, epot (105 B);
# the displacement test and the overlap search read pos and one older
# position (48 B); list phases add the 4-byte entries they must read.  The
# cell sort reads a position and writes a cell index and a cell entry per
# slot (32 B).  A GCMC trial reads the positions of the atoms in the 27 cells
# around its point (24 B each; the cell volume is bounded below by
# (rc + skin)^3, so the count is a lower bound).
PHASE_KERNEL = {"integrate": ("ermak_a_kernel", "ion", 120.0),
                "force_pairs": ("scan_mode_kernel + force_scan_span_kernel / "
                                "force_scan_listed_kernel + force_exact_mixed_kernel", "ion", 24.0),
                "force_sum": ("force_touched_kernel + force_ref_kernel", "ion", 105.0),
                "test_update1": ("pbc_dispmax_kernel + dispmax_exact_kernel", "ion", 48.0),
                "overlap": ("overlap_count_kernel + overlap_comp_kernel", "ion", 48.0),
                "test_update2": ("pbc_dispmax_kernel + dispmax_exact_kernel", "ion", 48.0),
                "commit": ("commit_kernel", "ion", 1.0),
                "gcmc_cells": ("gcmc_prep_kernel + gcmc_bin_kernel", "slot", 32.0),
                "gcmc": ("gcmc_pre_kernel + gcmc_fast_kernel", "trial", 24.0),
                "rho_piston": ("calc_rho_kernel", "ion", 48.0)}
# The roofline line reports the integrator (one kernel, the largest share of
# the step's launch list); the other phases are listed with their times.
ROOFLINE_PHASE = "integrate"
LIST_PHASES = ("force_pairs", "overlap")

def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """Barrier and max over ranks (gloo; the ranks run independent replicas)."""

    def __init__(self, ws):
        self.ws = ws
        self.pg = None
        if ws > 1:
            import torch.distributed as tdist

            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            tdist.init_process_group("gloo")
            self.tdist = tdist

    def barrier(self):
        if self.ws > 1:
            self.tdist.barrier()

    def reduce(self, x, op="max"):
        if self.ws == 1:
            return x
        import torch

        t = torch.tensor([float(x)], dtype=torch.float64)
        self.tdist.all_reduce(t, op=self.tdist.ReduceOp.MAX if op == "max" else self.tdist.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.tdist.destroy_process_group()


def job_value(dist, n_ion, steps, ms):
    """Whole-job particle-steps/s over all ranks: every rank's mobile ions x
    steps over the slowest rank's time `ms` (milliseconds).  Returns it
    with that time."""
    ms_max = dist.reduce(ms, "max")
    return dist.reduce(n_ion, "sum") * steps / (ms_max / 1e3), ms_max


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi during a region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv,noheader,nounits", "-lms",
                 "200", "-i", str(self.idx)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic(kernel_phase):
    """Per-launch DRAM bytes of the dominant kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        d = json.load(open(path))
        return d.get(kernel_phase)
    except (OSError, ValueError):
        return None


class Workload:
    """One benchmark system: parameters, per-replica values and atoms."""

    def __init__(self, name, rank, n_rep):
        import dml
        from tests import systems

        self.name = name
        if name == "c5":
            self.batched = True
            self.p, self.reps, self.atoms = systems.c5_batch(n_rep, seed=11 + 1000 * rank)
            self.n_electrode = 2 * systems.C5_CELLS ** 2 * 2 * n_rep
            self.desc = ("config 5: %d replicas x (40x40x2-cell bcc Li electrode, 6400 atoms, "
                         "+ 20000 Li+), 140.4x140.4x300 A, GCMC reservoir z in [200,300] with "
                         "%d trials/step, Ermak dt=1fs, skin 2" % (n_rep, self.p.nadj))
        elif name == "c4":
            self.batched = True
            self.p, self.reps, self.atoms = systems.c4_batch(n_rep, seed=13 + 1000 * rank)
            self.n_electrode = sum(int((a["z"] == dml.Z_CG).sum()) for a in self.atoms)
            self.desc = ("config 4: %d replicas of uneven size (L x L x 2-cell bcc Li electrode, "
                         "L uniform in 5..40; ions log-uniform in 50..20000; height by the 1 M "
                         "rule, at least 20 A), Brownian dt=5e-5 ps, skin 2, piston at half "
                         "height" % n_rep)
        elif name == "c2":
            self.batched = False
            self.p = systems.c2_params(seed=1234 + rank)
            self.reps = None
            self.atoms = [systems.c2_atoms(seed=7 + rank)]
            self.n_electrode = 80000
            self.desc = ("config 2: 200k Li+ over an 80k-atom bcc Li electrode, 351x351x320 A, "
                         "Ermak dt=1fs, piston z0=160, skin 10")
        else:
            raise ValueError(name)
        self.n_rep = len(self.atoms)
        self.n_ion = sum(int((a["z"] != dml.Z_CG).sum()) for a in self.atoms)

    def config(self, ws):
        """The `config` object of both arms' lines (the same workload)."""
        return {"workload": self.desc, "replicas": self.n_rep, "n_ion": self.n_ion,
                "n_electrode": self.n_electrode,
                "parallelism": "replicas" if ws > 1 else "single",
                "l2": "GPU arm: not flushed, the K timed steps run as one K-step graph and "
                      "every step reads and writes more than %.1f GB of per-atom state, far "
                      "larger than the 129 MB L2; value_l2_flushed flushes before each step); "
                      "CPU reference arm: no flush" % (state_bytes(self) / 1e9)}

    def params(self, precision):
        import ctypes

        import dml

        q = dml.Params()
        ctypes.memmove(ctypes.byref(q), ctypes.byref(self.p), ctypes.sizeof(q))
        q.precision = precision
        return q

    def replica_params(self, r, precision):
        """Parameters of replica r alone (its box, planes and seed)."""
        p = self.params(precision)
        if self.batched:
            q = self.reps[r]
            p.box[:] = list(q.box)
            p.z0, p.zmax, p.z1, p.seed = q.z0, q.zmax, q.z1, q.seed
        return p

    scan_lanes = 0  # force scan lanes per row (0: autotuned)

    def open(self, precision, replicas=None):
        """A loaded context (all replicas, or the listed ones one by one)."""
        import dml

        p = self.params(precision)
        if not self.batched:
            sim = dml.Simulation(p)
            sim.set_atoms(self.atoms[0])
        else:
            idx = list(range(self.n_rep)) if replicas is None else replicas
            if len(idx) == 1:
                sim = dml.Simulation(self.replica_params(idx[0], precision))
                sim.set_atoms(self.atoms[idx[0]])
            else:
                sim = dml.Simulation(p, replicas=[self.reps[i] for i in idx])
                sim.set_atoms([self.atoms[i] for i in idx])
        if self.scan_lanes:
            sim.set_scan_lanes(self.scan_lanes)
        return sim


def timed_steps(sim, args, clocks=None):
    """W untimed steps, then K steps queued as one K-step CUDA graph (what
    dml_step does for a run of K steps), bracketed by one pair of CUDA events.
    No L2 flush: every step reads and writes more per-atom state than the L2
    holds (state_bytes)."""
    sim.set_graph_steps(max(1, args.steps))
    sim.step(args.warmup)
    c0 = sim.counters()
    if clocks:
        clocks.start()
    ms = sim.time_run(args.steps)
    clk = clocks.stop() if clocks else None
    c1 = sim.counters()
    return ms, c0, c1, clk


def flushed_steps(sim, args):
    """K more steps, each its own one-step graph between CUDA events, the L2
    flushed (256 MiB write) before each, outside the events."""
    c0 = sim.counters()
    ms = sim.time_steps(args.steps, flush_l2=True)
    c1 = sim.counters()
    return ms, c0, c1


def rebuild_window(sim, steps=500):
    """A longer window in which the replicas' neighbour lists are rebuilt as
    the atoms move (about every 40-50 steps per config-5 replica, at
    different steps in different replicas): graphs of 100 steps, one pair of
    CUDA events around the window."""
    sim.set_graph_steps(100)
    c0 = sim.counters()
    ms = sim.time_run(steps)
    c1 = sim.counters()
    n_ion = 0.5 * (c0["n_ref"] + c1["n_ref"])
    return {"value": n_ion * steps / (ms / 1e3), "unit": UNIT, "steps": steps,
            "ms_per_step": ms / steps,
            "list_builds": c1["list_builds"] - c0["list_builds"],
            "replica_rebuilds": c1["nupd"] - c0["nupd"]}


def state_bytes(wl):
    """A lower bound of the per-atom device state a step reads or writes
    (bytes): per mobile ion at least 200 B (the integrator alone reads 120 B
    of position, velocity, acceleration and element and writes position,
    FP32 copy, old position and noise; the force, displacement and overlap
    passes add more), per electrode atom 32 B (the displacement test's two
    FP32 positions)."""
    return int(wl.n_ion * 200 + wl.n_electrode * 32)


def force_error_probe(wl, nrep=4, steps=20):
    """Mixed vs FP64 forces on identical positions: replica r runs `steps`
    plain steps and one more ermak_a (the move that brings ions inside each
    other's r0), then that state is loaded into one context of each form and
    both run test_update and fuerza at those positions.  Relative error per
    mobile ion: |F_mixed - F_fp64|
    / max(|F_fp64|, F_rms), F_rms the RMS force of the ions that interact
    (ions with no pair inside r0 have exactly zero force in both forms); also
    the absolute error and the relative error of the total energy."""
    import numpy as np

    import dml

    EV = 96.485 * 100.0  # ui per eV (dana.F90:23)
    rel, rel_all, absd, emix, epl, inter = [], [], [], 0.0, 0.0, 0
    fmag, unfl = [], []
    for r in range(min(nrep, wl.n_rep)):
        sp = wl.open(dml.PRECISION_FP64, replicas=[r])
        sp.setup()
        sp.step(steps)
        sp.ermak_a(sp.counters()["step"] + 1)
        st = sp.get_atoms(replica=0) if wl.batched else sp.get_atoms()
        sp.close()
        out = []
        for prec in (dml.PRECISION_MIXED, dml.PRECISION_FP64):
            s = dml.Simulation(wl.replica_params(r, prec))
            s.set_atoms(st)
            s.test_update()
            s.fuerza()
            a = s.get_atoms()
            out.append((a["force"], a["epot"], a["z"]))
            s.close()
        (fm, em, z), (fp, ep, _) = out
        mob = z != dml.Z_CG
        fr = np.sqrt((fp[mob] ** 2).sum(1))
        d = np.sqrt(((fm[mob] - fp[mob]) ** 2).sum(1))
        hit = fr > 0
        inter += int(hit.sum())
        absd.append(d)
        if hit.any():
            frms = float(np.sqrt((fr[hit] ** 2).mean()))
            rel.append(d / np.maximum(fr, frms))
            rel_all.append(d / np.maximum(fr, float(np.sqrt((fr ** 2).mean()))))
            fmag.append(fr[hit])
            unfl.append(d[hit] / fr[hit])
        emix += float(em.sum())
        epl += float(ep.sum())
    e = np.concatenate(rel) if rel else np.zeros(1)
    ea = np.concatenate(rel_all) if rel_all else np.zeros(1)
    # |dF| / |F| with no floor, by decile of |F| over the interacting ions
    deciles = []
    if fmag:
        fm_all, un_all = np.concatenate(fmag), np.concatenate(unfl)
        order = np.argsort(fm_all)
        for part in np.array_split(order, 10):
            if len(part):
                deciles.append({"f_min_ev_per_A": float(fm_all[part].min() / EV),
                                "f_max_ev_per_A": float(fm_all[part].max() / EV),
                                "ions": int(len(part)),
                                "max_rel": float(un_all[part].max()),
                                "median_rel": float(np.median(un_all[part]))})
    return {"max_rel": float(e.max()), "rms_rel": float(np.sqrt((e ** 2).mean())),
            "unfloored": {"max_rel": float(max((x["max_rel"] for x in deciles), default=0.0)),
                          "by_force_decile": deciles},
            "max_rel_floor_all_ions": float(ea.max()),
            "max_abs_ev_per_A": float(np.concatenate(absd).max() / EV) if absd else 0.0,
            "energy_rel": float(abs(emix - epl) / abs(epl)) if epl else 0.0,
            "interacting_ions": inter, "replicas": min(nrep, wl.n_rep),
            "state": "after %d FP64 steps and an FP64 ermak_a, fuerza in both forms at those "
                     "positions" % steps,
            "tolerance": 1e-6, "within": bool(e.max() <= 1e-6)}


def deposition_probe(n_rep=64, steps=2000, cell_factor=1.0):
    """Deposition statistics of the two forms over seeds: n_rep config-1
    systems (400-atom bcc electrode, 200 Li+, piston), each its own ion
    placement and Philox seed, run `steps` Ermak steps in one batch per form.
    The captures per replica are compared: the chosen form's mean against the
    plain FP64 form's mean and spread over seeds.  The chosen form runs with
    cell edges of cell_factor x (rc + skin) (the cell size the autotuner
    picked for the timed workload); the plain form keeps the reference's."""
    import statistics as st

    import dml
    from tests import systems

    p = systems.c1_params(seed=500)
    reps = [dml.replica_of(p, seed=500 + 7919 * r) for r in range(n_rep)]
    atoms = [systems.c1_atoms(seed=900 + r) for r in range(n_rep)]
    depo = {}
    for form, prec in (("fp64", dml.PRECISION_FP64), ("mixed", dml.PRECISION_MIXED)):
        q = dml.Params()
        ctypes.memmove(ctypes.byref(q), ctypes.byref(p), ctypes.sizeof(q))
        q.precision = prec
        sim = dml.Simulation(q, replicas=reps)
        sim.set_atoms(atoms)
        sim.setup()
        if form == "mixed" and cell_factor != 1.0:
            sim.set_cell_factor(cell_factor)
        sim.step(steps)
        depo[form] = [int(sim.counters(replica=r)["depo"]) for r in range(n_rep)]
        sim.close()
    mf, mm = st.mean(depo["fp64"]), st.mean(depo["mixed"])
    sf = st.stdev(depo["fp64"])
    return {"system": "config 1 (10x10x2-cell electrode, 200 Li+, piston z0=30, Ermak dt=1fs)",
            "seeds": n_rep, "steps": steps, "mixed_cell_factor": cell_factor,
            "fp64_mean": mf, "fp64_sigma": sf,
            "mixed_mean": mm, "mixed_sigma": st.stdev(depo["mixed"]),
            "mean_difference_in_fp64_sigma": (mm - mf) / sf if sf else None,
            "within_1_sigma": bool(sf == 0.0 or abs(mm - mf) <= sf)}


def cpu_baseline_sample(wl, budget_s=12.0, max_steps=200, warmup=0):
    """Oracle (serial CPU restatement) on replica 0 of the workload, plain FP64;
    `warmup` untimed steps after setup."""
    import dml
    from tests import oracle_lib

    p = wl.params(dml.PRECISION_FP64)
    if wl.batched:
        r = wl.reps[0]
        p.box[:] = list(r.box)
        p.z0, p.zmax, p.z1, p.seed = r.z0, r.zmax, r.z1, r.seed
    o = oracle_lib.Oracle(p)
    o.set_atoms(wl.atoms[0])
    o.setup()
    if warmup > 0:
        o.step(warmup)
    n_ion0 = o.counters()["n_ref"]
    t0 = time.perf_counter()
    steps = 0
    while steps < max_steps:
        o.step(1)
        steps += 1
        if time.perf_counter() - t0 > budget_s and steps >= 2:
            break
    dt = time.perf_counter() - t0
    n_ion1 = o.counters()["n_ref"]
    return 0.5 * (n_ion0 + n_ion1) * steps / dt, steps, dt


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_reference_sample(wl, threads, budget_s, max_steps, warmup):
    """The oracle (serial CPU restatement, plain FP64) on `threads` replicas
    of the workload at once, one per host thread: ctypes releases the GIL
    for every oracle call and the oracle keeps no shared state.  Each thread
    sets up its replica and runs `warmup` untimed steps; then all start
    together and step until `max_steps` or the `budget_s` window ends.
    Returns the particle-steps/s of all threads together (mean mobile-ion
    count x steps, summed, over the wall time until the last one stopped),
    the steps per replica, the wall time and the atoms held."""
    import dml
    from tests import oracle_lib

    n = min(threads, len(wl.atoms))
    gate = threading.Barrier(n + 1)
    out = [None] * n
    errors = []

    def run(r):
        try:
            p = wl.params(dml.PRECISION_FP64)
            if wl.batched:
                rep = wl.reps[r]
                p.box[:] = list(rep.box)
                p.z0, p.zmax, p.z1, p.seed = rep.z0, rep.zmax, rep.z1, rep.seed
            o = oracle_lib.Oracle(p)
            o.set_atoms(wl.atoms[r])
            o.setup()
            if warmup > 0:
                o.step(warmup)
            n0 = o.counters()["n_ref"]
        except Exception as e:  # reported after the gate opens
            errors.append(e)
            gate.wait()
            return
        gate.wait()
        t0 = time.perf_counter()
        steps = 0
        while steps < max_steps:
            o.step(1)
            steps += 1
            if time.perf_counter() - t0 > budget_s and steps >= 2:
                break
        out[r] = (0.5 * (n0 + o.counters()["n_ref"]) * steps, steps, time.perf_counter())

    pool = [threading.Thread(target=run, args=(r,)) for r in range(n)]
    for t in pool:
        t.start()
    gate.wait()
    t0 = time.perf_counter()
    for t in pool:
        t.join()
    if errors:
        raise errors[0]
    dt = max(x[2] for x in out) - t0
    return (sum(x[0] for x in out) / dt, min(x[1] for x in out), dt, n,
            sum(len(a["z"]) for a in wl.atoms[:n]))


def run_reference(args, ws, rank):
    """The oracle timed on this host's cores, one replica of the workload per
    host thread."""
    if rank != 0:
        return 0
    wl = Workload(args.workload, 0, args.replicas)
    k = min(args.steps, 60)
    v, steps, dt, nthr, natoms = cpu_reference_sample(wl, host_threads(), budget_s=60.0,
                                                     max_steps=k, warmup=args.warmup)
    sample = ("%s; oracle on %d replicas at once, one per host thread (%d atoms in all), %d "
              "timed steps each after setup and %d warm-up steps"
              % (wl.desc, nthr, natoms, steps, args.warmup))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws,
            "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": wl.config(ws), "form": "plain FP64 (CPU oracle)",
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": nthr, "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def roofline_of(sim, wl, nprof):
    """The integrator's roofline in profiled steps (the graph's kernels
    launched one by one, CUDA events at the phase boundaries): its
    algorithmic bytes per launch / its device time per step, with every
    phase's time per step."""
    import dml

    ph = sim.profile_steps(nprof, flush_l2=True)
    c = sim.counters()
    n_ion = c["n_ref"]
    nn_mean = None
    try:
        nn, _ = sim.get_neighbors(sim.params.mnb, replica=0 if wl.batched else None)
        nn_mean = float(nn.mean())
    except Exception:  # noqa: BLE001
        pass
    dom = ROOFLINE_PHASE
    t_launch = ph[dom] / nprof / 1e3  # s per step of this phase
    kernel, unit, per = PHASE_KERNEL[dom]
    if dom == "integrate" and sim.params.integrator == dml.INTEGRATOR_BROWNIAN:
        kernel = "brownian_kernel"
    if unit == "ion":
        units = n_ion
    elif unit == "slot":
        units = wl.n_ion + wl.n_electrode
    else:
        p = sim.params
        rho = wl.n_ion / (wl.n_rep * p.box[0] * p.box[1] * (p.box[2] - 15.0))
        per = 24.0 * 27.0 * rho * (p.rc + p.skin) ** 3
        units = p.nadj * wl.n_rep
    byts = per * units
    if dom in LIST_PHASES and nn_mean:
        byts += 4.0 * nn_mean * n_ion
    peak, peak_kind = measured_peaks()
    achieved = byts / t_launch / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": ncu_traffic(wl.name + ":" + dom),
            "kernel": kernel, "kernel_phase": dom, "peak_source": peak_kind,
            "algorithmic_bytes_per_launch": byts, "bytes_unit": unit,
            "bytes_per_unit": per, "units_per_launch": units,
            "phase_ms_per_step": {k: v / nprof for k, v in ph.items()}}


def force_error_at(p, state, step):
    """Mixed vs FP64 forces at the positions reached by one FP64 ermak_a from
    `state` (the move brings ions inside each other's r0): both forms run
    test_update and fuerza on identical positions.  Metrics as in
    force_error_probe."""
    import copy

    import numpy as np

    import dml

    EV = 96.485 * 100.0
    q = copy.copy(p)
    q.precision = dml.PRECISION_FP64
    s0 = dml.Simulation(q)
    s0.set_atoms(state)
    s0.test_update()
    s0.ermak_a(step)
    moved = s0.get_atoms()
    s0.close()
    out = []
    for prec in (dml.PRECISION_MIXED, dml.PRECISION_FP64):
        q = copy.copy(p)
        q.precision = prec
        s1 = dml.Simulation(q)
        s1.set_atoms(moved)
        s1.test_update()
        s1.fuerza()
        a = s1.get_atoms()
        out.append((a["force"], a["epot"], a["z"]))
        s1.close()
    (fm, em, z), (fp, ep, _) = out
    mob = z != dml.Z_CG
    fr = np.sqrt((fp[mob] ** 2).sum(1))
    dd = np.sqrt(((fm[mob] - fp[mob]) ** 2).sum(1))
    hit = fr > 0
    frms = float(np.sqrt((fr[hit] ** 2).mean())) if hit.any() else 1.0
    rel = dd / np.maximum(fr, frms)
    return {"max_rel": float(rel.max()), "rms_rel": float(np.sqrt((rel[hit] ** 2).mean()))
            if hit.any() else 0.0, "max_abs_ev_per_A": float(dd.max() / EV),
            "energy_rel": float(abs(em.sum() - ep.sum()) / abs(ep.sum())) if ep.sum() else 0.0,
            "interacting_ions": int(hit.sum())}


def run_accuracy(args):
    """Config 3: config 2's system (80k electrode atoms, 200k Li+) in the
    chosen form against the plain FP64 form (bit-exact to the oracle): the
    force and energy error at steps 0, 1/10 and all of the run (seed 0), and
    the deposition count of each form over `--seeds` seeds (Philox streams
    keyed by seed, step and atom, shared by both forms)."""
    import copy
    import statistics as st

    import dml
    from tests import systems

    dml.build()
    steps = args.steps
    marks = [0, steps // 10, steps]
    errors, depo = {}, {"fp64": [], "mixed": []}
    rate = {"fp64": [], "mixed": []}
    for seed in range(args.seeds):
        p = systems.c2_params(seed=1234 + seed)
        atoms = systems.c2_atoms(seed=7 + seed)
        sims = {}
        for form, prec in (("fp64", dml.PRECISION_FP64), ("mixed", dml.PRECISION_MIXED)):
            q = copy.copy(p)
            q.precision = prec
            sims[form] = dml.Simulation(q)
            sims[form].set_atoms(atoms)
            sims[form].setup()
        done = 0
        for m in marks:
            if m > done:
                for form, sim in sims.items():
                    c0 = sim.counters()
                    t0 = time.perf_counter()
                    sim.step(m - done)
                    dt = time.perf_counter() - t0
                    c1 = sim.counters()
                    rate[form].append(0.5 * (c0["n_ref"] + c1["n_ref"]) * (m - done) / dt)
                done = m
            if seed == 0:
                st_fp = sims["fp64"].get_atoms()
                errors[str(m)] = force_error_at(p, st_fp, sims["fp64"].counters()["step"] + 1)
        for form, sim in sims.items():
            depo[form].append(int(sim.counters()["depo"]))
            sim.close()
    mf, mm = st.mean(depo["fp64"]), st.mean(depo["mixed"])
    sf = st.stdev(depo["fp64"]) if len(depo["fp64"]) > 1 else 0.0
    diff = [a - b for a, b in zip(depo["mixed"], depo["fp64"])]
    line = {"metric": METRIC, "workload": "config 3: config 2's system (351x351x320 A, 80k "
            "electrode atoms + 200k Li+, Ermak dt=1fs, piston z0=160, skin 10) in the chosen "
            "form vs the plain FP64 form", "steps": steps, "seeds": args.seeds,
            "value": st.mean(rate["mixed"]), "unit": UNIT,
            "plain_fp64_value": st.mean(rate["fp64"]),
            "value_note": "wall-clock particle-steps/s of the runs below (step() calls, "
                          "including list rebuilds)",
            "force_error_at_step": errors, "force_error_tolerance": 1e-6,
            "deposition": {"fp64": depo["fp64"], "mixed": depo["mixed"],
                           "fp64_mean": mf, "fp64_sigma": sf, "mixed_mean": mm,
                           "mean_difference_in_fp64_sigma": (mm - mf) / sf if sf else None,
                           "per_seed_difference": diff,
                           "within_1_sigma": bool(sf == 0.0 or abs(mm - mf) <= sf)},
            "data": "synthetic", "dtype": "f32 pair forces, int64 fixed-point sums, f64 positions"}
    print(json.dumps(line), flush=True)
    return 0


def run_gpu(args, ws, rank, local):
    import dml

    dml.build()
    dist = Dist(ws)
    wl = Workload(args.workload, rank, args.replicas)
    wl.scan_lanes = args.scan_lanes
    form = args.form or ("chosen" if wl.batched else "plain")
    prec = dml.PRECISION_MIXED if form == "chosen" else dml.PRECISION_FP64
    clocks = Clocks(local)

    # The chosen form's cell size is picked by the autotuner (edge bound
    # 1.0 .. 1.5 x (rc + skin), timed over 10 steps each) on a context of its
    # own, so that the measured run starts from the same state as the others.
    cell_tuning = None
    if form == "chosen" and wl.batched:
        tune = wl.open(prec)
        tune.setup()
        tune.tune_cells(steps=10)
        cell_tuning = tune.cell_tuning()
        tune.close()

    # Main arm: the whole workload in one context.
    sim = wl.open(prec)
    sim.setup()
    if cell_tuning and cell_tuning["factor"] != 1.0:
        sim.set_cell_factor(cell_tuning["factor"])
    dist.barrier()
    ms, c0, c1, clk = timed_steps(sim, args, clocks)
    dist.barrier()
    n_ion = 0.5 * (c0["n_ref"] + c1["n_ref"])
    value, ms_max = job_value(dist, n_ion, args.steps, ms)
    # the same rate counting every atom, frozen electrode atoms included
    value_all, _ = job_value(dist, 0.5 * (c0["n_atoms"] + c1["n_atoms"]), args.steps, ms)
    # the same steps one graph each, the L2 flushed before each
    ms_f, f0, f1 = flushed_steps(sim, args)
    value_flushed, _ = job_value(dist, 0.5 * (f0["n_ref"] + f1["n_ref"]), args.steps, ms_f)
    per_step, per_rebuild = sim.launches_per_step()
    tuning = sim.tuning()
    if cell_tuning:
        tuning["cells"] = cell_tuning
    launches = per_step * args.steps + per_rebuild * (c1["list_builds"] - c0["list_builds"])
    roofline = roofline_of(sim, wl, max(3, min(args.steps, 10)))
    counters = {k: c1[k] - c0[k] for k in ("choques", "depo", "try_", "choques3", "gcmc_ins",
                                           "gcmc_del", "list_builds")}
    counters["n_ref"] = c1["n_ref"]
    with_rebuilds = rebuild_window(sim) if not args.no_compare else None
    sim.close()

    # Comparison arms (chosen form only): the same batch in plain FP64, and
    # replicas run one per context in plain FP64 (the reference's way: one
    # system per run).
    compare = None
    if form == "chosen" and not args.no_compare:
        compare = {}
        compare["force_error"] = force_error_probe(wl)
        compare["deposition"] = deposition_probe(
            cell_factor=cell_tuning["factor"] if cell_tuning else 1.0)
        sp = wl.open(dml.PRECISION_FP64)
        sp.setup()
        ms_p, p0, p1, _ = timed_steps(sp, args)
        np_ion = 0.5 * (p0["n_ref"] + p1["n_ref"])
        compare["plain_fp64_batched"] = {"value": np_ion * args.steps / (ms_p / 1e3),
                                         "ms_per_step": ms_p / args.steps,
                                         "depo": p1["depo"] - p0["depo"]}
        sp.close()
        tot_ion_steps, tot_s = 0.0, 0.0
        nsolo = min(wl.n_rep, 4)
        for r in range(nsolo):
            s1 = wl.open(dml.PRECISION_FP64, replicas=[r])
            s1.setup()
            ms_1, q0, q1, _ = timed_steps(s1, args)
            tot_ion_steps += 0.5 * (q0["n_ref"] + q1["n_ref"]) * args.steps
            tot_s += ms_1 / 1e3
            s1.close()
        solo = tot_ion_steps / tot_s
        compare["plain_fp64_one_replica_per_context"] = {
            "value": solo, "replicas_timed": nsolo,
            "ms_per_step_per_replica": 1e3 * tot_s / nsolo / args.steps}
        compare["speedup_vs_plain_one_per_context"] = value / dist.reduce(solo, "sum") * 1.0
        compare["speedup_vs_plain_batched"] = value / compare["plain_fp64_batched"]["value"]

    # End to end through the C ABI with host buffers.
    e2e = None
    if rank == 0 and not args.no_e2e:
        h2d = sum(a["pos"].nbytes + a["z"].nbytes for a in wl.atoms)
        t0 = time.perf_counter()
        s2 = wl.open(prec)
        s2.setup()
        if cell_tuning and cell_tuning["factor"] != 1.0:  # the cell size the tuner picked
            s2.set_cell_factor(cell_tuning["factor"])
        done, d2h = 0, 0
        while done < args.steps:
            k = min(NWR, args.steps - done)
            s2.step(k)
            done += k
            for out in s2.get_atoms_batch(fields=("pos", "z")):
                d2h += out["pos"].nbytes + out["z"].nbytes
            d2h += ctypes.sizeof(dml.Observables) * len(s2.salida())
        t1 = time.perf_counter()
        s2.close()
        e2e = {"value": n_ion * args.steps / (t1 - t0), "unit": UNIT,
               "h2d_bytes_per_step": h2d / args.steps, "d2h_bytes_per_step": d2h / args.steps,
               "wall_s": t1 - t0}

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        v, k, dt = cpu_baseline_sample(wl)
        cpu = {"value": v, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": "oracle (serial C++ restatement, plain FP64) on replica 0 of the same "
                         "workload (%d atoms): %d steps after setup in %.1f s"
                         % (len(wl.atoms[0]["z"]), k, dt)}
    dist.close()
    if rank != 0:
        return 0
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "value_including_electrode": value_all,
            "value_l2_flushed": {"value": value_flushed, "unit": UNIT,
                                 "ms_per_step": ms_f / args.steps,
                                 "how": "the next K steps, one graph launch each, the L2 "
                                        "flushed before each step outside the events"},
            "value_with_rebuilds": with_rebuilds,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 pair forces, int64 fixed-point sums, f64 integration" if form == "chosen"
            else "f64",
            "data": "synthetic",
            "config": wl.config(ws),
            "form": ("chosen: mixed precision, %d replicas in every launch" % wl.n_rep)
            if form == "chosen" else "plain FP64 (bit-exact to the oracle)",
            "autotuner": tuning,
            "clocks": clk, "e2e": e2e, "gpu_launches": launches, "roofline": roofline,
            "cpu_baseline": cpu, "compare": compare, "counters": counters}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="c5", choices=["c5", "c2", "c3", "c4"])
    ap.add_argument("--seeds", type=int, default=8)
    ap.add_argument("--replicas", type=int, default=None)
    ap.add_argument("--form", default=None, choices=["chosen", "plain"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-compare", action="store_true")
    ap.add_argument("--scan-lanes", type=int, default=0,
                    help="pin the force scan's lanes per list row (profiling a reduced "
                         "workload with the full workload's mapping); 0: autotuned")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 10000 if args.workload == "c3" else 100
    if args.replicas is None:
        args.replicas = 1024 if args.workload == "c4" else 256
    if args.warmup < 3:
        args.warmup = 3
    ws, rank, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, ws, rank)
    if args.workload == "c3":
        return run_accuracy(args) if rank == 0 else 0
    if ws > 1 and "CUDA_VISIBLE_DEVICES" not in os.environ:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    return run_gpu(args, ws, rank, local)


if __name__ == "__main__":
    sys.exit(main())
