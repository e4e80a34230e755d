"""The N > 1 path of bench.py on CPU: world_size-2 gloo ranks (replicas
only: each rank advances its own realizations; the only collectives are the
barrier and the max-over-ranks of the timed region)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
mp = pytest.importorskip("torch.multiprocessing")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, ws, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(ws), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import bench
    w, r, local = bench.dist_env()
    dist = bench.dist_init(w)
    bench.barrier(dist)
    m = bench.max_over_ranks(dist, 10.0 + r)  # the slowest rank's time wins
    seeds = bench.replica_seeds(r, 4)
    got = [None] * w
    dist.all_gather_object(got, seeds)
    out[r] = (w, m, got)
    dist.destroy_process_group()


def test_two_gloo_ranks_time_max_and_disjoint_seeds():
    port = _free_port()
    with mp.Manager() as man:
        out = man.dict()
        mp.spawn(_rank_main, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    for r in (0, 1):
        w, m, seeds = res[r]
        assert w == 2 and m == 11.0
        assert not set(seeds[0]) & set(seeds[1])


def test_reference_arm_other_ranks_exit_without_work(monkeypatch):
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    assert bench.run_reference(None) == 0  # returns before reading args or the device
