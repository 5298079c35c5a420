"""The multi-rank path of bench.py on CPU (gloo, world size 2).

Ranks run independent replica batches: no collective touches the data
path.  bench.py only needs a barrier, the max of the ranks' times and the
sum of their ion counts (Dist, job_value), different seeds per rank, and a
reference arm that prints from rank 0 alone under torchrun.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

torch = pytest.importorskip("torch")
mp = pytest.importorskip("torch.multiprocessing")


def free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(ws), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    dist = bench.Dist(ws)
    dist.barrier()
    # rank r: (r + 1) * 1000 ions timed in (r + 1) * 10 ms over 5 steps
    value, ms_max = bench.job_value(dist, (rank + 1) * 1000.0, 5, (rank + 1) * 10.0)
    wl = bench.Workload("c5", rank, 2)
    seeds = [int(r.seed) for r in wl.reps]
    first_ion = wl.atoms[0]["pos"][-1].tolist()
    dist.barrier()
    dist.close()
    with open(os.path.join(out_dir, "rank%d.json" % rank), "w") as f:
        json.dump({"value": value, "ms_max": ms_max, "seeds": seeds, "ion": first_ion}, f)


def test_two_gloo_ranks_reduce_and_shard(tmp_path):
    ws = 2
    mp.start_processes(_rank_main, args=(ws, free_port(), str(tmp_path)), nprocs=ws,
                       join=True, start_method="spawn")
    res = [json.load(open(tmp_path / ("rank%d.json" % r))) for r in range(ws)]
    for r in res:
        # (1000 + 2000) ions x 5 steps over the slower rank's 20 ms
        assert r["ms_max"] == 20.0
        assert r["value"] == pytest.approx(3000.0 * 5 / 0.020)
    # weak scaling: each rank builds its own replicas (seeds and placements)
    assert not set(res[0]["seeds"]) & set(res[1]["seeds"])
    assert res[0]["ion"] != res[1]["ion"]


def test_reference_arm_under_torchrun_prints_from_rank0_only():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), "bench.py",
           "--impl", "reference", "--gpus", "2", "--steps", "3", "--warmup", "3",
           "--replicas", "4"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    p = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, p.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["warmup"] == 3
    assert d["value"] > 0 and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["value"] == d["value"]


def test_reference_arm_maps_only_the_oracle_library():
    """The reference arm builds its workload (parameters, electrode, ion
    placement) and steps it without the CUDA library: the process maps
    oracle/_build/liboracle.so and nothing of din-mol-li_gb300/."""
    code = ("import argparse, sys; sys.path.insert(0, '.'); import bench; "
            "a = argparse.Namespace(workload='c5', replicas=2, steps=2, warmup=3); "
            "bench.run_reference(a, 1, 0); "
            "m = open('/proc/self/maps').read(); "
            "print('MAPS', int('liboracle.so' in m), int('libdml.so' in m))")
    p = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True,
                       timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    line = [l for l in p.stdout.splitlines() if l.startswith("{")][0]
    d = json.loads(line)
    assert d["config"]["replicas"] == 2 and d["config"]["n_ion"] == 40000
    assert p.stdout.splitlines()[-1] == "MAPS 1 0"
