"""Replica runs over two CPU processes (`gloo`): the split of modes and cosmologies over ranks,
the max-over-ranks timing and the gather of per-rank results.  The per-rank work in the last case
is the oracle's perturbation solve of that rank's modes, standing in for the GPU solve; the
gathered sources must equal a single-process solve of all modes."""
import json
import os
import socket

import numpy as np
import pytest

from symboltz import replicas as R

MODEL5 = dict(lmax_g=5, lmax_nu=5, lmax_h=5, nx=4, Hswitch=1, Heswitch=6, reionization=1)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir, case):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    r, w = R.init("gloo")
    assert (r, w) == (rank, world)
    res = {}
    if case == "collectives":
        R.barrier()
        res["max"] = R.reduce_over_ranks([1.0 + rank, -rank], op="max")
        res["sum"] = R.reduce_over_ranks([1.0 + rank], op="sum")
        res["throughput"] = list(R.throughput(units_per_rank=100 * (rank + 1), seconds_per_rank=2.0 + rank))
        costs = np.array([800, 200, 650, 410, 300, 790, 220, 505])
        mine = R.shard_by_cost(costs, rank, world)
        res["gathered"] = R.gather_rows(np.stack([mine, costs[mine] * 3], axis=1), mine).tolist()
    else:
        import oracle as O
        bg = O.Background(O.PLANCK18, MODEL5)
        ks = np.geomspace(3.0, 300.0, 6)
        taus = np.linspace(0.05, 0.9 * bg.tau0, 12)
        lo, hi = R.shard(len(ks), rank, world)
        src, st, _ = bg.solve_pt(ks[lo:hi], 1e-4, taus, mode=0)
        res["status"] = np.asarray(st).tolist()
        np.save(os.path.join(out_dir, f"gathered{rank}.npy"), R.gather_rows(src, np.arange(lo, hi)))
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump(res, f)
    R.finalize()


def _run(case, tmp_path, world=2):
    import torch.multiprocessing as mp
    mp.start_processes(_worker, args=(world, _free_port(), str(tmp_path), case), nprocs=world, join=True,
                       start_method="spawn")
    return [json.load(open(tmp_path / f"rank{r}.json")) for r in range(world)]


def test_shard_tiles_the_range():
    for n in (0, 1, 5, 1000, 1001):
        for world in (1, 2, 3, 8):
            parts = [R.shard(n, r, world) for r in range(world)]
            assert parts[0][0] == 0 and parts[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(parts, parts[1:]))
            sizes = [hi - lo for lo, hi in parts]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        R.shard(10, 2, 2)


def test_shard_by_cost_balances_and_covers():
    rng = np.random.default_rng(0)
    costs = rng.integers(200, 801, size=256)
    for world in (1, 2, 4, 8):
        owned = [R.shard_by_cost(costs, r, world) for r in range(world)]
        allidx = np.sort(np.concatenate(owned))
        np.testing.assert_array_equal(allidx, np.arange(len(costs)))
        loads = [costs[o].sum() for o in owned]
        assert max(loads) - min(loads) <= costs.max()


def test_single_process_is_the_identity():
    assert R.rank_world() == (0, 1) or "WORLD_SIZE" in os.environ
    assert R.reduce_over_ranks([3.0, 4.0]) == [3.0, 4.0]
    rate, units, t = R.throughput(10, 2.0)
    assert (rate, units, t) == (5.0, 10.0, 2.0)
    np.testing.assert_array_equal(R.gather_rows(np.array([[2], [0], [1]]), [2, 0, 1]), [[0], [1], [2]])


def test_two_ranks_collectives(tmp_path):
    res = _run("collectives", tmp_path)
    for r in res:
        assert r["max"] == [2.0, 0.0]
        assert r["sum"] == [3.0]
        assert r["throughput"] == [300.0 / 3.0, 300.0, 3.0]  # all units over the slowest rank
        costs = np.array([800, 200, 650, 410, 300, 790, 220, 505])
        np.testing.assert_array_equal(np.array(r["gathered"]), np.stack([np.arange(8), costs * 3], axis=1))


def test_two_ranks_sharded_modes_equal_one_solve(tmp_path):
    import oracle as O
    res = _run("modes", tmp_path)
    assert all(s == 0 for r in res for s in r["status"])
    bg = O.Background(O.PLANCK18, MODEL5)
    ks = np.geomspace(3.0, 300.0, 6)
    taus = np.linspace(0.05, 0.9 * bg.tau0, 12)
    full, st, _ = bg.solve_pt(ks, 1e-4, taus, mode=0)
    assert np.all(np.asarray(st) == 0)
    for r in range(2):
        np.testing.assert_array_equal(np.load(tmp_path / f"gathered{r}.npy"), full)
