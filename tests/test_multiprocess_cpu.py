"""The N > 1 host path of bench.py on CPU: two gloo ranks on 127.0.0.1.

* the barrier and the max over ranks (timing is the slowest rank's);
* batch instances shard across ranks with every instance on exactly one
  rank (no data-path collective);
* the reference arm runs on rank 0 only; other ranks return without work;
* a rank that raises leaves the other rank's collective with an error
  instead of a hang (short process-group timeout);
* `bench.py --gpus 2` started without a launcher starts its two ranks itself
  (torch.distributed.run on 127.0.0.1), and rank 0 prints one line for both.
"""
import json
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir, mode):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port),
                       "RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    from qcs_gb300 import workloads as W
    res = {"rank": rank}
    if mode == "normal":
        d = bench.Dist()
        d.barrier()
        res["max"] = d.max(float(10 + rank))
        inst = W.variational_batch(37, seed=3)
        mine = bench.shard(inst, d)
        res["mine"] = [i for i, x in enumerate(inst) if any(x is y for y in mine)]

        class A:  # the reference arm's arguments
            qubits, depth, seed, cpu_sample_gates, warmup, steps, gpus = 12, 2, 1, 4, 0, 1, world
        res["reference_returned"] = bench.run_reference(A, d) is None if rank != 0 else None
        d.close()
    else:  # rank 1 fails before the collective; rank 0 must see an error
        import datetime
        import torch.distributed as td
        td.init_process_group("gloo", timeout=datetime.timedelta(seconds=5))
        if rank == 1:
            os._exit(3)
        import torch
        try:
            td.all_reduce(torch.ones(1))
            res["error"] = None
        except Exception as e:  # noqa: BLE001 - any collective error is the point
            res["error"] = type(e).__name__
    with open(os.path.join(out_dir, f"r{rank}.json"), "w") as f:
        json.dump(res, f)


def _spawn(tmp_path, mode):
    port = _free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, str(tmp_path), mode))
             for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        if p.is_alive():
            p.kill()
            pytest.fail("rank did not finish")
    return [json.load(open(tmp_path / f"r{r}.json")) for r in range(2)
            if (tmp_path / f"r{r}.json").exists()]


def test_two_gloo_ranks_barrier_max_and_shards(tmp_path):
    res = _spawn(tmp_path, "normal")
    assert len(res) == 2
    assert res[0]["max"] == res[1]["max"] == 11.0
    a, b = set(res[0]["mine"]), set(res[1]["mine"])
    assert not (a & b) and a | b == set(range(37))
    assert res[1]["reference_returned"] is True


def test_a_failed_rank_ends_the_other_ranks_collective_with_an_error(tmp_path):
    res = _spawn(tmp_path, "fail")
    assert len(res) == 1 and res[0]["rank"] == 0
    assert res[0]["error"] is not None


def test_bench_gpus_2_starts_two_ranks():
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = {k: v for k, v in os.environ.items()
           if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK", "MASTER_ADDR", "MASTER_PORT")}
    p = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--gpus", "2",
                        "--workload", "shards", "--instances", "37"],
                       capture_output=True, text=True, timeout=300, env=env, cwd=root)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, p.stdout[-2000:]  # rank 0 alone prints
    out = json.loads(lines[0])
    assert out["n_gpus"] == 2
    ranks = out["ranks"]
    assert [r["rank"] for r in ranks] == [0, 1]
    assert ranks[0]["pid"] != ranks[1]["pid"]  # two processes ran
    a, b = set(ranks[0]["instances"]), set(ranks[1]["instances"])
    assert not (a & b) and a | b == set(range(37))
