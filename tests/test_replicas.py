"""The N > 1 path of bench.py (independent replicas, one process per GPU):
its torch.distributed plumbing on CPU with world_size 2 over gloo --
barrier, max over ranks of the step time, and the reference arm printing one
line from rank 0 while rank 1 exits without work."""
import json
import os
import pathlib
import socket
import subprocess
import sys

ROOT = pathlib.Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _run_ranks(args: list, world: int = 2, timeout: int = 300) -> list:
    port = _free_port()
    procs = []
    for rank in range(world):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable] + args, cwd=ROOT, env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    out = []
    for p in procs:
        so, se = p.communicate(timeout=timeout)
        assert p.returncode == 0, se[-2000:]
        out.append(so)
    return out


def test_max_over_ranks_and_barrier_gloo():
    code = ("import bench\n"
            "world, rank, local, pg = bench.dist_setup()\n"
            "v = bench.max_over_ranks(pg, 10.0 * (rank + 1))\n"
            "bench.barrier(pg)\n"
            "print('RESULT', rank, world, v)\n"
            "pg.destroy_process_group()\n")
    outs = _run_ranks(["-c", code])
    got = sorted(line.split()[1:] for o in outs for line in o.splitlines() if line.startswith("RESULT"))
    assert got == [["0", "2", "20.0"], ["1", "2", "20.0"]]


def test_reference_arm_prints_from_rank0_only(native_lib):
    outs = _run_ranks(["bench.py", "--impl", "reference", "--workload", "commit", "--gpus", "2", "--steps", "1",
                       "--warmup", "0"])
    lines = [[l for l in o.splitlines() if l.startswith("{")] for o in outs]
    assert len(lines[0]) == 1 and lines[1] == []
    d = json.loads(lines[0][0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
