"""The multi-GPU host path (independent replicas, one process per GPU) on CPU:
two gloo ranks over 127.0.0.1 run the timing collectives bench.py uses (the
max over ranks of the timed region, the units every rank processed), and the
reference arm under torchrun prints one line from rank 0 only."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      WORLD_SIZE=str(world), RANK=str(rank), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    from meshlesshydro_gb300 import replicas
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ws, r, local = replicas.dist_env()
        seconds = [0.25, 0.75][rank]
        units = [1000, 3000][rank]
        res = {"env": [ws, r, local],
               "seed": replicas.replica_seed(2, r),
               "t": replicas.job_seconds(seconds, dist),
               "units": replicas.gather_units(units, dist)}
        res["rate"] = replicas.job_rate(res["units"], res["t"])
        dist.barrier()
    finally:
        dist.destroy_process_group()
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump(res, f)


def test_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    port = free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(2)]
    for r in range(2):
        assert res[r]["env"] == [2, r, r]
        assert res[r]["seed"] == 2 + r                 # every replica its own initial conditions
        assert res[r]["t"] == 0.75                     # the slowest rank's time, on every rank
        assert res[r]["units"] == [1000.0, 3000.0]     # every rank's units, in rank order
        assert res[r]["rate"] == pytest.approx(4000 / 0.75)


def test_single_process_needs_no_collective():
    from meshlesshydro_gb300 import replicas
    assert replicas.job_seconds(1.5, None) == 1.5
    assert replicas.gather_units(7, None) == [7.0]
    assert replicas.job_rate([7.0], 0.5) == 14.0


def test_reference_arm_prints_from_rank_zero_only():
    """bench.py --impl reference under torchrun with two ranks: rank 0 times
    the CPU arm (the restatement on the host's threads, its serial rate
    beside) and prints one JSON line; rank 1 exits 0 without work."""
    port = free_port()
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", str(port),
                        os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "kh100",
                        "--steps", "1", "--warmup", "0"],
                       capture_output=True, text=True, timeout=300, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["value"] > 0 and line["e2e"]["value"] == line["value"]
    assert line["cpu_baseline"]["cores"] >= 1 and line["cpu_baseline"]["kind"] == "port"
    assert line["cpu_baseline"]["serial_value"] > 0
