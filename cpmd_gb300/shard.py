"""State-block partition of the band loop over ranks.

The reference splits the states of rhoofr/vpsi over "CP groups": group p of P
owns the contiguous block given by part_1d_nbr_el_in_blk / part_1d_get_el_in_blk
(part_1d.mod.F90:21-56: the first mod(n, P) groups get one extra state), pairs
are formed inside the block (rhoofr_utils.mod.F90:306-310), and one sum over the
groups completes the density (cp_grp_redist, cp_grp_utils.mod.F90:98-120;
rhoofr_utils.mod.F90:457-459) and C2 (vpsi_utils.mod.F90:710).

On GB300 a cell is one GPU's work and the benchmark runs replicas, so nothing
here moves data between GPUs by itself; these are the host-side pieces a
multi-GPU run uses: the block of a rank and the density/energy reduction over
a torch.distributed group (NCCL on GPUs, gloo on CPUs).
"""
from __future__ import annotations


def state_block(nstate: int, rank: int, world: int) -> tuple[int, int]:
    """[first, last) states owned by `rank` of `world` (part_1d block partition)."""
    res = nstate % world
    nbr = nstate // world + (1 if rank < res else 0)
    first = rank * (nstate // world) + min(rank, res)
    return first, first + nbr


def rhoofr_sharded(rhoofr, c0, f, rank: int, world: int, group=None):
    """Density and kinetic energy of all states from per-rank blocks.

    ``rhoofr(c0_block, f_block) -> (rho, ekin, ...)`` is the local band loop
    (a :class:`cpmd_gb300.Context` method, or any stand-in with that shape);
    ``c0`` is (ngw, nstate) column-major (numpy) or (nstate, ngw) (torch).
    Returns (rho, ekin) summed over the group.
    """
    import numpy as np
    import torch
    import torch.distributed as dist
    is_torch = isinstance(c0, torch.Tensor)
    n = int(c0.shape[0] if is_torch else c0.shape[1])
    s0, s1 = state_block(n, rank, world)
    blk = c0[s0:s1] if is_torch else np.asfortranarray(c0[:, s0:s1])
    out = rhoofr(blk, f[s0:s1])
    rho, ekin = out[0], out[1]
    if world > 1:
        t = rho if is_torch else torch.from_numpy(np.ascontiguousarray(rho))
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
        e = torch.tensor([ekin], dtype=torch.float64, device=t.device)
        dist.all_reduce(e, op=dist.ReduceOp.SUM, group=group)
        rho = t if is_torch else t.numpy()
        ekin = float(e.item())
    return rho, ekin
