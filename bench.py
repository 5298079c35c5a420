#!/usr/bin/env python3
"""Benchmark of din-mol-Li's per-step hot path on GB300.

Workload (config 2 of the benchmark set): a 351 x 351 x 320 Å box, a frozen
bcc Li electrode of 100 x 100 x 4 cells (80 000 atoms) and 200 000 mobile
Li+ ions placed uniformly in z in [15, 300) Å with 2.5 Å minimum separation
(seeded synthetic data: the reference measures no dataset).  Ermak
integrator, dt = 1 fs, piston reservoir with z0 = 160 Å, skin 10 Å.  A step
is one iteration of the reference's loop body (src/dana.F90:173-265):
ermak_a, fuerza, ermak_b, test_update, overlap_moveback, test_update,
capture commit, calc_rho, maxz -- all on the device, plain FP64 form,
bit-exact to the oracle.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line.  `value` = mobile-ion steps per second over all ranks
(device time, inputs resident, L2 flushed between steps).  `e2e` = the same
metric through the C ABI with host arrays: upload, setup, K steps with a
positions download every 100 steps (the reference's output cadence) and the
final download, wall clock.  `--impl reference` times the CPU restatement of
the reference (oracle/) on this host; rank 0 only.
"""
import argparse
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

METRIC = "particle-steps/s on 1 GB300: mixed+batched vs plain FP64 at force err ≤1e-6"
UNIT = "particle-steps/s"
N_ION, N_CG = 200000, 80000
NWR = 100  # output cadence of the reference's tests (entrada.ini nwr)

# Algorithmic bytes per mobile ion and step, FP64 state touched once
# (integrate: read pos, vel, acel, write pos, old_cg = 120 B; force + ermak_b:
# read pos 24, vel, acel, element 49, write vel, acel 48, epot 8 = 129 B);
# list-scanning phases add the 4-byte list entries they must read.
PHASE_BYTES_PER_ION = {"integrate": 120.0, "force_pairs": 24.0, "force_sum": 105.0,
                       "test_update1": 48.0, "overlap": 48.0, "test_update2": 48.0,
                       "commit": 1.0, "rho_piston": 48.0}
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


def make_system(seed):
    import dml
    from tests import systems

    p = systems.c2_params(seed=1234 + seed)
    atoms = systems.c2_atoms(seed=7 + seed)
    return p, atoms


def cpu_baseline_sample(p, atoms, budget_s=12.0, max_steps=200):
    """Oracle (serial CPU restatement) on the same system: steps after setup."""
    from tests import oracle_lib

    o = oracle_lib.Oracle(p)
    o.set_atoms(atoms)
    o.setup()
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


def run_reference(args, ws, rank):
    if rank != 0:
        return 0
    p, atoms = make_system(0)
    from tests import oracle_lib

    o = oracle_lib.Oracle(p)
    o.set_atoms(atoms)
    o.setup()
    o.step(min(args.warmup, 3))
    k = min(args.steps, 60)
    n0 = o.counters()["n_ref"]
    t0 = time.perf_counter()
    o.step(k)
    dt = time.perf_counter() - t0
    n1 = o.counters()["n_ref"]
    v = 0.5 * (n0 + n1) * k / dt
    sample = "config 2 system (80k electrode + 200k ions), %d timed steps after setup" % k
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws,
            "steps": k, "warmup": min(args.warmup, 3), "ms_per_step": 1e3 * dt / k,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": "config 2: 200k Li+ over an 80k-atom bcc Li electrode, Ermak, "
                                   "piston", "n_ion": N_ION, "n_electrode": N_CG},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": 1, "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_gpu(args, ws, rank, local):
    import numpy as np

    import dml

    dml.build()
    dist = Dist(ws)
    p, atoms = make_system(rank)
    sim = dml.Simulation(p)
    sim.set_atoms(atoms)
    sim.setup()
    sim.step(args.warmup)
    n_ion0 = sim.counters()["n_ref"]
    clocks = Clocks(local)
    dist.barrier()
    clocks.start()
    nupd0 = sim.counters()["nupd"]
    ms = sim.time_steps(args.steps, flush_l2=True)
    clk = clocks.stop()
    dist.barrier()
    c = sim.counters()
    n_ion = 0.5 * (n_ion0 + c["n_ref"])
    ms_max = dist.reduce(ms, "max")
    ions_all = dist.reduce(n_ion, "sum")
    value = ions_all * args.steps / (ms_max / 1e3)
    per_step, per_rebuild = sim.launches_per_step()
    launches = per_step * args.steps + per_rebuild * (c["nupd"] - nupd0)

    # Per-phase device times (same work, un-graphed) for the roofline.
    nprof = max(3, min(args.steps, 20))
    ph = sim.profile_steps(nprof, flush_l2=True)
    nn_mean = None
    try:
        nn, _ = sim.get_neighbors(p.mnb)
        nn_mean = float(nn.mean())
    except Exception:  # noqa: BLE001
        pass
    dom = max(ph, key=ph.get)
    t_launch = ph[dom] / nprof / 1e3  # s per step of this phase
    byts = PHASE_BYTES_PER_ION[dom] * n_ion
    if dom in LIST_PHASES and nn_mean:
        byts += 4.0 * nn_mean * n_ion
    peak, peak_kind = measured_peaks()
    achieved = byts / t_launch / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": ncu_traffic(dom), "kernel_phase": dom,
                "peak_source": peak_kind,
                "phase_ms_per_step": {k: v / nprof for k, v in ph.items()}}
    sim.close()

    # End to end through the C ABI with host buffers.
    e2e = None
    if rank == 0 and not args.no_e2e:
        pos_bytes = atoms["pos"].nbytes + atoms["z"].nbytes
        t0 = time.perf_counter()
        s2 = dml.Simulation(p)
        s2.set_atoms(atoms)
        s2.setup()
        done, d2h = 0, 0
        n_atoms = len(atoms["z"])
        while done < args.steps:
            k = min(NWR, args.steps - done)
            s2.step(k)
            done += k
            out = s2.get_atoms(n_atoms)
            d2h += out["pos"].nbytes + out["z"].nbytes
        t1 = time.perf_counter()
        s2.close()
        e2e = {"value": n_ion * args.steps / (t1 - t0), "unit": UNIT,
               "h2d_bytes_per_step": pos_bytes / args.steps, "d2h_bytes_per_step": d2h / args.steps,
               "wall_s": t1 - t0}

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        v, k, dt = cpu_baseline_sample(p, atoms)
        cpu = {"value": v, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": "oracle (serial C++ restatement) on the same system: %d steps after "
                         "setup in %.1f s" % (k, dt)}
    dist.close()
    if rank != 0:
        return 0
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "config 2: 200k Li+ over an 80k-atom bcc Li electrode, "
                                   "351x351x320 A, Ermak dt=1fs, piston z0=160, skin 10",
                       "form": "plain FP64 (bit-exact to the oracle)", "n_ion": N_ION,
                       "n_electrode": N_CG, "parallelism": "replicas" if ws > 1 else "single",
                       "l2": "flushed between steps (256 MiB write outside the timed events)"},
            "clocks": clk, "e2e": e2e, "gpu_launches": launches, "roofline": roofline,
            "cpu_baseline": cpu, "counters": {k: c[k] for k in ("nupd", "choques", "depo", "try_",
                                                                 "choques3", "n_ref")}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    ws, rank, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, ws, rank)
    if ws > 1 and "CUDA_VISIBLE_DEVICES" not in os.environ:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    return run_gpu(args, ws, rank, local)


if __name__ == "__main__":
    sys.exit(main())
