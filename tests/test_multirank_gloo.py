"""World-size-2 host logic on CPU (gloo): the benchmark's replica timing
(barrier, max over ranks) and the state-block density reduction."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _init(rank, world, port):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    return dist


def _bench_worker(rank, world, port, q):
    dist = _init(rank, world, port)
    import bench
    bench.barrier(world)
    q.put((rank, bench.allreduce_max(1.5 + rank, world)))
    dist.destroy_process_group()


def _shard_worker(rank, world, port, q):
    dist = _init(rank, world, port)
    from cpmd_gb300.shard import rhoofr_sharded
    from cpmd_gb300.synth import make_small_cell
    from oracle import cpmd_oracle as O
    cl = make_small_cell(10.26, 16, 6.0, 7, seed=21)
    b = cl.basis

    def local(c, f):
        return O.rhoofr(c, f, b.mill, b.nr, b.kr, b.omega, b.hg, b.tpiba2, b.geq0)
    rho, ekin = rhoofr_sharded(local, cl.c0, cl.f, rank, world)
    q.put((rank, rho, ekin))
    dist.destroy_process_group()


def _run(fn, world=2):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=fn, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    return sorted(out, key=lambda t: t[0])


def test_state_block_partition():
    from cpmd_gb300.shard import state_block
    for n in (1, 7, 16, 33):
        for w in (1, 2, 3, 5):
            blocks = [state_block(n, r, w) for r in range(w)]
            assert blocks[0][0] == 0 and blocks[-1][1] == n
            assert all(blocks[i][1] == blocks[i + 1][0] for i in range(w - 1))
            sizes = [e - s for s, e in blocks]
            assert max(sizes) - min(sizes) <= 1 and sizes == sorted(sizes, reverse=True)


def test_bench_replica_reduction_gloo():
    out = _run(_bench_worker)
    assert [v for _, v in out] == [2.5, 2.5]


def test_sharded_density_gloo():
    from cpmd_gb300.synth import make_small_cell
    from oracle import cpmd_oracle as O
    out = _run(_shard_worker)
    cl = make_small_cell(10.26, 16, 6.0, 7, seed=21)
    b = cl.basis
    rho, ekin, _, _ = O.rhoofr(cl.c0, cl.f, b.mill, b.nr, b.kr, b.omega, b.hg, b.tpiba2, b.geq0)
    for _, r, e in out:
        assert np.abs(r - rho).max() <= 1e-12 * np.abs(rho).max()
        assert abs(e - ekin) <= 1e-12 * ekin
