"""Grid sharding across ranks (one GPU per rank) and the single reduction.

E_xc, V_xc = dE_xc/dD and dE_xc/dtheta are all sums over grid points
(functional.py:316-342), so the path shards by contiguous grid slices: every
rank holds the replicated density matrix, parameters and basis, evaluates its
own slice, and one all-reduce of the packed (E, V, dtheta) finishes the step.
There is no other exchange.
"""
from __future__ import annotations

import dataclasses
from typing import Sequence, Tuple

import torch

_GRID_FIELDS_2D = ("ao",)


def grid_slice(n_grid: int, rank: int, world: int, granule: int = 128) -> Tuple[int, int]:
    """Contiguous, balanced [start, stop) of rank's points; boundaries on `granule` where the size allows."""
    if not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of {world}")
    units = (n_grid + granule - 1) // granule
    base, extra = divmod(units, world)
    u0 = rank * base + min(rank, extra)
    u1 = u0 + base + (1 if rank < extra else 0)
    return min(u0 * granule, n_grid), min(u1 * granule, n_grid)


def shard_molecule(mol, rank: int, world: int):
    """The molecule restricted to rank's grid slice (per-point arrays sliced; D, h1e, ... replicated)."""
    a, b = grid_slice(int(mol.grid.weights.shape[0]), rank, world)
    grid = dataclasses.replace(mol.grid, weights=mol.grid.weights[a:b],
                               coords=None if mol.grid.coords is None else mol.grid.coords[a:b])
    g2 = mol.grad_n_ao
    if isinstance(g2, dict):
        g2 = {k: v[a:b] for k, v in g2.items()}
    elif g2 is not None:
        g2 = g2[a:b]
    ehf = None if mol.ehf is None else mol.ehf[..., a:b]
    chi = None if getattr(mol, "chi", None) is None else mol.chi[a:b]  # chi is (grid, omega, spin, orbitals)
    return dataclasses.replace(mol, grid=grid, ao=mol.ao[a:b], grad_ao=mol.grad_ao[a:b], grad_n_ao=g2, ehf=ehf,
                               chi=chi, _resident=None)


def allreduce_sum(tensors: Sequence[torch.Tensor], group=None) -> list:
    """Sum every tensor over the ranks in place, with one collective (packed into one buffer)."""
    import torch.distributed as dist

    flat = torch.cat([t.reshape(-1) for t in tensors])
    dist.all_reduce(flat, op=dist.ReduceOp.SUM, group=group)
    off = 0
    for t in tensors:
        n = t.numel()
        t.copy_(flat[off:off + n].view_as(t))
        off += n
    return list(tensors)


def xc_energy_and_grads_sharded(functional, params, molecule, want_dparams: bool = False, group=None):
    """(E_xc, V_xc[, dE_xc/dtheta]) of the whole grid: this rank evaluates its slice
    (shard_molecule), one all-reduce sums the parts.  ``molecule`` is the full,
    replicated description; its per-point arrays are sliced, never copied whole
    to the device.  With ``want_dparams`` the functional is a NeuralFunctional
    and the parameter gradient tree (views of one flat vector) is summed too."""
    import torch.distributed as dist

    rank, world = dist.get_rank(group), dist.get_world_size(group)
    part = shard_molecule(molecule, rank, world)
    if want_dparams:
        e, v, dp = functional.xc_energy_and_grads_params(params, part)
        leaves = [t for mod in dp["params"].values() for t in mod.values()]
        allreduce_sum([e.reshape(1), v] + leaves, group)
        return e, v, dp
    e, v = functional.xc_energy_and_grads(params, part)
    allreduce_sum([e.reshape(1), v], group)
    return e, v
