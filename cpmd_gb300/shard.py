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


def _allreduce_sum(t, group=None):
    """Sum over the group in place; gloo reduces host tensors, so a CUDA tensor
    goes through a host copy there (NCCL reduces it where it is)."""
    import torch
    import torch.distributed as dist
    if t.is_cuda and dist.get_backend(group) == "gloo":
        h = t.cpu()
        dist.all_reduce(h, op=dist.ReduceOp.SUM, group=group)
        t.copy_(h)
    else:
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t


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
        _allreduce_sum(t, group)
        e = torch.tensor([ekin], dtype=torch.float64)
        dist.all_reduce(e, op=dist.ReduceOp.SUM, group=group)
        rho = t if is_torch else t.numpy()
        ekin = float(e.item())
    return rho, ekin


def vpsi_sharded(vpsi, c0, c2, f, vpot, rank: int, world: int, group=None):
    """C2 of all states from per-rank blocks: each rank applies ``vpsi(c0_block,
    c2_block, f_block, vpot)`` to its own states in place, and one sum over the
    group of the otherwise zero blocks completes C2 on every rank, the
    reference's cp_grp_redist of C2 (vpsi_utils.mod.F90:710).  c0, c2 as in
    :func:`rhoofr_sharded`; c2 is accumulated like vpsi's."""
    import numpy as np
    import torch
    is_torch = isinstance(c0, torch.Tensor)
    n = int(c0.shape[0] if is_torch else c0.shape[1])
    s0, s1 = state_block(n, rank, world)
    if is_torch:
        part = torch.zeros_like(c2)
        blk = c2[s0:s1].clone()
        vpsi(c0[s0:s1], blk, f[s0:s1], vpot)
        part[s0:s1] = blk - c2[s0:s1]
        if world > 1:
            _allreduce_sum(part, group)
        c2 += part
        return c2
    part = np.zeros_like(c2)
    blk = np.asfortranarray(c2[:, s0:s1].copy())
    vpsi(np.asfortranarray(c0[:, s0:s1]), blk, f[s0:s1], vpot)
    part[:, s0:s1] = blk - c2[:, s0:s1]
    if world > 1:
        t = torch.from_numpy(np.ascontiguousarray(part))
        _allreduce_sum(t, group)
        part = t.numpy()
    c2 += part
    return c2


def g_block(ngw: int, rank: int, world: int) -> tuple[int, int]:
    """[first, last) plane waves of `rank` when C is split by G rows (G = 0 on rank 0)."""
    return state_block(ngw, rank, world)


def overlap_sharded(c0, ngw: int, rank: int, world: int, geq0: bool = True, group=None, stream=None):
    """The Γ overlap S (n x n) of states split by G rows: each rank forms the
    partial 2 Re(C_r^H C_r) of its plane waves (the G = 0 term on the rank that
    holds it) with the allocation-free overlap kernel, and one sum of S over the
    group completes it -- the S allreduce of a G-split ortho (n^2 doubles per
    step instead of moving C).  ``c0`` is a CUDA tensor (nstate, ldc) complex128."""
    import ctypes as C
    import torch
    from . import _lib
    lib = _lib.load()
    n, ldc = int(c0.shape[0]), int(c0.shape[1])
    g0, g1 = g_block(ngw, rank, world)
    s = torch.zeros((n, n), dtype=torch.float64, device=c0.device)
    if g1 > g0:
        base = c0.data_ptr() + 16 * g0
        st = stream if stream is not None else (torch.cuda.current_stream().cuda_stream or 1)
        rc = lib.gbcp_ovlap_noalloc(C.c_void_p(base), ldc, g1 - g0, n, 1 if (geq0 and g0 == 0) else 0,
                                    C.c_void_p(s.data_ptr()), C.c_void_p(st))
        if rc != 0:
            raise _lib.GbcpError("gbcp_ovlap_noalloc", rc)
    if world > 1:
        _allreduce_sum(s, group)
    return s
