"""World-size-2 host logic (gloo): the benchmark's replica timing (barrier,
max over ranks), the state-block density and C2 reductions on CPU with the
oracle as each rank's band loop, and (-m gpu) the same with the CUDA context
as the band loop plus the G-split overlap reduction, both ranks on cuda:0."""
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


def _vpsi_worker(rank, world, port, q):
    dist = _init(rank, world, port)
    from cpmd_gb300.shard import vpsi_sharded
    from cpmd_gb300.synth import make_small_cell
    from oracle import cpmd_oracle as O
    cl = make_small_cell(10.26, 16, 6.0, 7, seed=22)
    b = cl.basis

    def local(c, c2, f, v):
        c2[:] = O.vpsi(c, c2, f, v, b.mill, b.nr, b.hg, b.tpiba2, b.geq0)
    c2 = np.zeros_like(cl.c0)
    vpsi_sharded(local, cl.c0, c2, cl.f, cl.vpot, rank, world)
    q.put((rank, c2))
    dist.destroy_process_group()


def test_sharded_vpsi_gloo():
    """Each rank applies vpsi to its state block; one sum over the group gives every
    rank all of C2 (the reference's cp_grp_redist of C2)."""
    from cpmd_gb300.synth import make_small_cell
    from oracle import cpmd_oracle as O
    out = _run(_vpsi_worker)
    cl = make_small_cell(10.26, 16, 6.0, 7, seed=22)
    b = cl.basis
    ref = O.vpsi(cl.c0, np.zeros_like(cl.c0), cl.f, cl.vpot, b.mill, b.nr, b.hg, b.tpiba2, b.geq0)
    for _, c2 in out:
        assert np.abs(c2 - ref).max() <= 1e-12 * np.abs(ref).max()


def _cuda_worker(rank, world, port, q):
    """Both ranks on cuda:0 (separate processes, separate contexts, no kernel waits on
    the other rank): the CUDA Context as each rank's local band loop, and the G-split
    overlap through the allocation-free kernel."""
    dist = _init(rank, world, port)
    import torch
    from cpmd_gb300 import Context
    from cpmd_gb300.shard import overlap_sharded, rhoofr_sharded, vpsi_sharded
    from cpmd_gb300.synth import make_small_cell
    torch.cuda.set_device(0)
    cl = make_small_cell(10.26, 32, 20.0, 13, seed=23)
    b = cl.basis
    ctx = Context(b, "fp64")
    c0 = torch.from_numpy(np.ascontiguousarray(cl.c0.T)).cuda()
    f = torch.from_numpy(cl.f).cuda()
    v = torch.from_numpy(cl.vpot).cuda()

    def local_rho(c, ff):
        return ctx.rhoofr(c, ff)

    def local_vpsi(c, c2, ff, vv):
        ctx.vpsi(c, c2, ff, vv)
    rho, ekin = rhoofr_sharded(local_rho, c0, f, rank, world)
    c2 = torch.zeros_like(c0)
    vpsi_sharded(local_vpsi, c0, c2, f, v, rank, world)
    s = overlap_sharded(c0, b.ngw, rank, world, b.geq0)
    torch.cuda.synchronize()
    q.put((rank, rho.cpu().numpy(), ekin, np.asfortranarray(c2.cpu().numpy().T), s.cpu().numpy()))
    ctx.close()
    dist.destroy_process_group()


@pytest.mark.gpu
def test_sharded_band_loop_and_overlap_on_cuda_gloo():
    from cpmd_gb300.synth import make_small_cell
    from oracle import cpmd_oracle as O
    out = _run(_cuda_worker)
    cl = make_small_cell(10.26, 32, 20.0, 13, seed=23)
    b = cl.basis
    rho, ekin, _, _ = O.rhoofr(cl.c0, cl.f, b.mill, b.nr, b.kr, b.omega, b.hg, b.tpiba2, b.geq0)
    c2 = O.vpsi(cl.c0, np.zeros_like(cl.c0), cl.f, cl.vpot, b.mill, b.nr, b.hg, b.tpiba2, b.geq0)
    s = O.overlap(cl.c0, b.geq0)
    for _, r, e, c, sm in out:
        assert np.abs(r - rho).max() <= 1e-10 * np.abs(rho).max()
        assert abs(e - ekin) <= 1e-10 * ekin
        assert np.abs(c - c2).max() <= 1e-10 * np.abs(c2).max()
        assert np.abs(sm - s).max() <= 1e-12 * np.abs(s).max()
