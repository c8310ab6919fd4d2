"""The multi-rank path on CPU: two gloo ranks take their grid slices of one
Molecule through the library's sharding (shard_molecule inside
xc_energy_and_grads_sharded), evaluate each slice with the oracle (no GPU
here), and the library's one all-reduce reproduces the full-grid E_xc, V_xc
and dE/dtheta."""
import os
import tempfile

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from graddft_gb300 import sharding, synthetic


def test_grid_slices_cover_and_balance():
    for n, world in ((1000, 2), (4096, 4), (129, 3), (5, 2)):
        cuts = [sharding.grid_slice(n, r, world) for r in range(world)]
        assert cuts[0][0] == 0 and cuts[-1][1] == n
        assert all(cuts[i][1] == cuts[i + 1][0] for i in range(world - 1))
        sizes = [b - a for a, b in cuts]
        assert max(sizes) - min(sizes) <= 128
    with pytest.raises(ValueError):
        sharding.grid_slice(10, 2, 2)


class _OracleSliceFunctional:
    """Stands in for a NeuralFunctional on CPU ranks: evaluates the slice it is given with the oracle."""

    def xc_energy_and_grads_params(self, params, part):
        import oracle as O

        e, v, dp = O.xc_energy_and_grads("DM21", part.rdm1.numpy(), part.ao.numpy(), part.grad_ao.numpy(),
                                         part.grad_n_ao[2].numpy(), part.grid.weights.numpy(), params=params,
                                         ehf=part.ehf.numpy(), want_param_grads=True)
        tree = {"params": {k: {kk: torch.as_tensor(g) for kk, g in d.items()} for k, d in dp["params"].items()}}
        self.n_points = int(part.grid.weights.shape[0])
        return torch.tensor(e, dtype=torch.float64), torch.as_tensor(v), tree


def _inputs():
    import oracle as O

    wl = synthetic.make_workload(1000, 16, 3, seed=4, box_angstrom=6.0, centre_box_angstrom=4.0)
    ao, g1, g2 = O.eval_ao_planes(wl.basis, wl.coords)
    rho = np.einsum("sab,ra,rb->rs", wl.rdm1, ao, ao)
    ehf = synthetic.make_ehf(1000, 2, rho, 2)
    params = synthetic.glorot_params(layer_widths=(32, 32), seed=1)
    return wl, ao, g1, g2, ehf, params


def _rank(rank, world, port, path):
    import torch.distributed as dist

    from graddft_gb300 import Grid, Molecule

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    wl, ao, g1, g2, ehf, params = _inputs()
    t = lambda x: torch.as_tensor(np.asarray(x), dtype=torch.float64)  # noqa: E731
    mol = Molecule(grid=Grid(coords=t(wl.coords), weights=t(wl.weights)), atom_index=None, nuclear_pos=None,
                   ao=t(ao), grad_ao=t(g1), grad_n_ao={2: t(g2)}, rdm1=t(wl.rdm1), nuclear_repulsion=0.0,
                   h1e=None, vj=None, mo_coeff=None, mo_occ=None, mo_energy=None, rep_tensor=None, ehf=t(ehf))
    fn = _OracleSliceFunctional()
    e, v, dp = sharding.xc_energy_and_grads_sharded(fn, params, mol, want_dparams=True)
    a, b = sharding.grid_slice(1000, rank, world)
    assert fn.n_points == b - a  # each rank evaluated only its own slice
    leaves = [dp["params"][k][kk] for k in sorted(dp["params"]) for kk in sorted(dp["params"][k])]
    if rank == 0:
        np.savez(path, e=e.numpy(), v=v.numpy(), **{f"p{i}": t.numpy() for i, t in enumerate(leaves)})
    dist.destroy_process_group()


def test_two_rank_shard_and_reduce_matches_full_grid():
    import oracle as O

    path = os.path.join(tempfile.mkdtemp(), "sum.npz")
    port = 29500 + os.getpid() % 1000
    mp.start_processes(_rank, args=(2, port, path), nprocs=2, start_method="spawn")
    got = np.load(path)
    wl, ao, g1, g2, ehf, params = _inputs()
    e, v, dp = O.xc_energy_and_grads("DM21", wl.rdm1, ao, g1, g2, wl.weights, params=params, ehf=ehf,
                                     want_param_grads=True)
    assert abs(float(got["e"]) - e) <= 1e-12 * abs(e)
    assert np.max(np.abs(got["v"] - v)) <= 1e-12 * np.max(np.abs(v))
    leaves = [dp["params"][k][kk] for k in sorted(dp["params"]) for kk in sorted(dp["params"][k])]
    for i, g in enumerate(leaves):
        assert np.max(np.abs(got[f"p{i}"] - g)) <= 1e-11 * max(np.max(np.abs(g)), 1e-300), i
