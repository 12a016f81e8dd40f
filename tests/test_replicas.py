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


def test_reference_arm_reports_the_whole_host(capsys, monkeypatch):
    """Rank 0's reference line: one reference process per host core, `value` the
    median over the timed steps of the host's summed trajectories/s, the serial
    one-core figure beside it.  The samplers are replaced by fixed numbers."""
    import multiprocessing
    import statistics
    sys.path.insert(0, ROOT)
    import bench

    class Pool:
        def __init__(self, n):
            self.n = n

        def __enter__(self):
            return self

        def __exit__(self, *a):
            return False

    class Ctx:
        pass
    Ctx.Pool = Pool
    seen = []

    def host_sample(pool, cores, seconds, seed, iters_per_traj):
        seen.append((pool.n, cores, seed))
        assert iters_per_traj == 300 * bench.SOLVES_PER_TRAJ
        return 0.004 + 0.001 * len(seen), "reference"
    monkeypatch.setattr(multiprocessing, "get_context", lambda kind: Ctx)
    monkeypatch.setattr(bench, "host_cores", lambda: 4)
    monkeypatch.setattr(bench, "cpu_host_sample", host_sample)
    monkeypatch.setattr(bench, "host_iteration_count", lambda: 300)
    monkeypatch.setattr(bench, "cpu_sample",
                        lambda iters, repeats=1, count_source="": dict(value=0.001, kind="reference", cores=1,
                                                                       sample="one core"))

    class Args:
        steps, warmup, gpus = 3, 1, 1
    bench.run_reference(Args(), ws=1, rank=0)
    line = json.loads(capsys.readouterr().out.strip())
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC
    assert len(seen) == 4 and all(n == 4 and c == 4 for n, c, _ in seen)
    assert len({s for _, _, s in seen}) == 4                       # fresh fields every step
    assert line["value"] == pytest.approx(statistics.median([0.006, 0.007, 0.008]))
    assert line["cg_iterations"]["first_solve_counted_on_host"] == 300
    cb = line["cpu_baseline"]
    assert cb["cores"] == 4 and cb["value"] == line["value"] and cb["kind"] == "reference"
    assert cb["single_process"] == {"value": 0.001, "cores": 1, "kind": "reference", "sample": "one core"}
    assert line["e2e"] == {"value": line["value"], "unit": "trajectories/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
