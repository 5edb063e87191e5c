"""The multi-rank host logic (emix_gb300.replicas) on two gloo ranks on the CPU:
the barrier, the maximum and sum of the ranks' values, and the split of the
48-grid ensemble between ranks (every grid on exactly one rank, balanced)."""
import socket

import pytest

from emix_gb300 import fields as F
from emix_gb300 import replicas


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        replicas.barrier(world)
        mx = replicas.max_over_ranks(1.5 + rank, world, "cpu")
        sm = replicas.sum_over_ranks(1.0 + rank, world, "cpu")
        costs = [nx * ny * nz for nx, ny, nz in F.ensemble_shapes(48, 7)]
        mine = replicas.shard_by_cost(costs, world)[rank]
        cells = replicas.sum_over_ranks(sum(costs[i] for i in mine), world, "cpu")
        replicas.barrier(world)
        out.put((rank, mx, sm, mine, cells, sum(costs)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    for rank, mx, sm, mine, cells, total in res:
        assert mx == 2.5 and sm == 3.0
        assert cells == total            # the two shares cover the ensemble
    a, b = set(res[0][3]), set(res[1][3])
    assert not (a & b) and len(a | b) == 48


def test_ensemble_shapes_match_the_ensemble():
    shapes = F.ensemble_shapes(6, 7)
    ws = F.ensemble(ngrids=6, seed=7, only={1, 4})
    assert [(w.grid.nx, w.grid.ny, w.grid.nz) for w in ws] == [shapes[1], shapes[4]]


def test_shard_by_cost_balances_and_covers():
    costs = [nx * ny * nz for nx, ny, nz in F.ensemble_shapes(48, 7)]
    for world in (1, 2, 3, 8):
        parts = replicas.shard_by_cost(costs, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(48))
        loads = [sum(costs[i] for i in p) for p in parts]
        # LPT: no rank exceeds the mean by more than the largest item
        assert max(loads) - sum(costs) / world <= max(costs)
    with pytest.raises(ValueError):
        replicas.shard_by_cost(costs, 0)
