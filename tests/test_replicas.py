"""Multi-rank host logic (pyhub_gb300.replicas) on CPU: two gloo ranks.

Single-sector solves run as replicas and batched Green's-function sweeps
shard by cluster; what crosses ranks is bookkeeping only (barriers, the
maximum time, the sum of units).  These tests run that bookkeeping with
world_size 2 over gloo on 127.0.0.1."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, out_dir):
    os.environ.update({"WORLD_SIZE": str(ws), "RANK": str(rank), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import json
    from pyhub_gb300 import replicas as RP
    from pyhub_gb300.core import greens_batched as GB
    w = RP.init("gloo")
    clusters = GB.c4_clusters(11, seed=0)
    mine = RP.shard(list(range(len(clusters))), rank, ws)
    RP.barrier(sync_cuda=False)
    # rank r "processed" len(mine) clusters in (r+1) seconds
    rate, total, tmax = RP.aggregate_rate(len(mine), float(rank + 1))
    res = {"world": list(w), "mine": mine, "rate": rate, "total": total, "tmax": tmax,
           "max": RP.max_over_ranks(10.0 * rank), "sum": RP.sum_over_ranks(rank + 1)}
    RP.barrier(sync_cuda=False)
    RP.finish()
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump(res, f)


def test_two_gloo_ranks(tmp_path):
    import json
    import torch.multiprocessing as mp
    ws = 2
    port = _free_port()
    ctx = mp.start_processes(_rank_main, args=(ws, port, str(tmp_path)), nprocs=ws, join=False, start_method="spawn")
    while not ctx.join(timeout=120):
        pass
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(ws)]
    # the shards are disjoint and together cover every cluster
    assert sorted(res[0]["mine"] + res[1]["mine"]) == list(range(11))
    assert not set(res[0]["mine"]) & set(res[1]["mine"])
    for r in range(ws):
        assert res[r]["world"] == [2, r, r]
        assert res[r]["total"] == 11.0
        assert res[r]["tmax"] == 2.0          # the slowest rank's time
        assert res[r]["rate"] == pytest.approx(11.0 / 2.0)
        assert res[r]["max"] == 10.0
        assert res[r]["sum"] == 3.0


def test_single_rank_is_local():
    """Without a launcher the helpers are the identity (no process group)."""
    from pyhub_gb300 import replicas as RP
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        assert k not in os.environ or os.environ[k] in ("1", "0")
    assert RP.world()[0] == 1
    assert RP.shard([1, 2, 3], 0, 1) == [1, 2, 3]
    assert RP.aggregate_rate(6.0, 2.0) == (3.0, 6.0, 2.0)


def _cpu_sweep(specs, nw=64):
    """Host stand-in for the batched sweep (same result structure): the
    non-interacting G_ii(w) of each cluster's hopping matrix, shifted by U/2."""
    import numpy as np
    w = np.linspace(-10.0, 10.0, nw)
    out = {}
    for k, spec in enumerate(specs):
        ek, V = np.linalg.eigh(spec["t"])
        g = ((V ** 2)[None, :, :] / (w[:, None, None] - ek[None, None, :] - 0.5 * spec["U"] + 0.05j)).sum(axis=2)
        out[k] = {"e0": float(ek[: spec["N"]].sum()), "G": np.stack([g.T, g.T])}
    return out


def _gather_main(rank, ws, port, out_dir):
    os.environ.update({"WORLD_SIZE": str(ws), "RANK": str(rank), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import pickle
    from pyhub_gb300 import replicas as RP
    from pyhub_gb300.core import greens_batched as GB
    RP.init("gloo")
    clusters = GB.c4_clusters(9, seed=1)
    merged = GB.sharded_sweep(clusters, rank, ws, sweep_fn=_cpu_sweep)
    RP.barrier(sync_cuda=False)
    RP.finish()
    with open(os.path.join(out_dir, f"gather{rank}.pkl"), "wb") as f:
        pickle.dump(merged, f)


def test_sharded_sweep_gathers_every_cluster_on_rank0(tmp_path):
    """Two gloo ranks sweep disjoint halves of 9 clusters; rank 0 ends with
    every cluster's G(w), equal to a single-rank sweep of the same clusters."""
    import pickle
    import numpy as np
    import torch.multiprocessing as mp
    from pyhub_gb300.core import greens_batched as GB
    ws = 2
    port = _free_port()
    ctx = mp.start_processes(_gather_main, args=(ws, port, str(tmp_path)), nprocs=ws, join=False,
                             start_method="spawn")
    while not ctx.join(timeout=120):
        pass
    got = pickle.load(open(tmp_path / "gather0.pkl", "rb"))
    assert pickle.load(open(tmp_path / "gather1.pkl", "rb")) is None
    ref = _cpu_sweep(GB.c4_clusters(9, seed=1))
    assert sorted(got) == list(range(9))
    for c in range(9):
        assert got[c]["e0"] == ref[c]["e0"]
        assert np.array_equal(got[c]["G"], ref[c]["G"])
