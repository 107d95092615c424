"""The N > 1 path of bench.py: ranks are independent replicas (the search
does not shard), so the only exchange is the final reduction -- the slowest
rank's times and the sum of every rank's candidates. Run here as two gloo
ranks on the CPU; the reference arm does its work on rank 0 only."""
import json
import os
import socket
import sys

import torch.multiprocessing as mp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out: str):
    sys.path.insert(0, REPO)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r: device time r + 1, wall time 2(r + 1), 10(r + 1) candidates
        res = bench.reduce_over_ranks(rank + 1.0, 2.0 * (rank + 1), 10 * (rank + 1), "cpu")
        with open(f"{out}.{rank}", "w") as f:
            json.dump(res, f)
    finally:
        dist.destroy_process_group()


def test_replica_reduction_two_gloo_ranks(tmp_path):
    out = str(tmp_path / "res")
    mp.spawn(_rank, args=(2, _free_port(), out), nprocs=2, join=True)
    for r in range(2):
        with open(f"{out}.{r}") as f:
            t_dev, t_wall, cands = json.load(f)
        assert (t_dev, t_wall, cands) == (2.0, 4.0, 30.0)


def test_reference_arm_works_on_rank_zero_only(monkeypatch, capsys):
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--gpus", "2"])
    args = bench.parse()
    assert bench.run_reference(args) is None
    assert capsys.readouterr().out == ""
