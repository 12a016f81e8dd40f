"""The multi-GPU path of bench.py is replicas only: independent chains per
rank, no collective on the data path, a barrier around the timed region and
the maximum time over ranks.  Its host side runs here as two gloo ranks on the
CPU (no GPU needed)."""
import json
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2", RANK=str(rank),
                      LOCAL_RANK=str(rank), BENCH_BACKEND="gloo")
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist
    ws, r, local = bench.dist_init()
    bench.barrier(ws)
    t = bench.allmax(ws, 1.5 + rank)           # the slower rank's time wins
    seed = bench.replica_seed(r)
    bench.barrier(ws)
    dist.destroy_process_group()
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump({"ws": ws, "rank": r, "local": local, "max": t, "seed": seed}, f)


def test_two_gloo_ranks(tmp_path):
    port = _free_port()
    mp.start_processes(_rank_main, args=(port, str(tmp_path)), nprocs=2, start_method="spawn", join=True)
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(2)]
    assert [r["rank"] for r in res] == [0, 1] and all(r["ws"] == 2 for r in res)
    assert all(r["max"] == 2.5 for r in res)
    assert res[0]["seed"] != res[1]["seed"]     # independent chains


def test_reference_arm_runs_on_rank0_only(capsys):
    sys.path.insert(0, ROOT)
    import bench

    class Args:
        steps, warmup, gpus = 1, 0, 2
    bench.run_reference(Args(), ws=2, rank=1)   # rank 1: no work, no output
    assert capsys.readouterr().out == ""
