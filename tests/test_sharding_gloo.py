"""The multi-rank path on CPU: two gloo ranks evaluate their grid slices with
the oracle and one all-reduce reproduces the full-grid E_xc, V_xc and dE/dtheta."""
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


def _rank(rank, world, port, path):
    import torch.distributed as dist

    import oracle as O

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    wl = synthetic.make_workload(1000, 16, 3, seed=4, box_angstrom=6.0, centre_box_angstrom=4.0)
    ao, g1, g2 = O.eval_ao_planes(wl.basis, wl.coords)
    rho = np.einsum("sab,ra,rb->rs", wl.rdm1, ao, ao)
    ehf = synthetic.make_ehf(1000, 2, rho, 2)
    params = synthetic.glorot_params(layer_widths=(32, 32), seed=1)
    a, b = sharding.grid_slice(1000, rank, world)
    e, v, dp = O.xc_energy_and_grads("DM21", wl.rdm1, ao[a:b], g1[a:b], g2[a:b], wl.weights[a:b], params=params,
                                     ehf=ehf[..., a:b], want_param_grads=True)
    leaves = [torch.as_tensor(dp["params"][k][kk]) for k in sorted(dp["params"]) for kk in sorted(dp["params"][k])]
    out = sharding.allreduce_sum([torch.tensor(e, dtype=torch.float64), torch.as_tensor(v)] + leaves)
    if rank == 0:
        np.savez(path, e=out[0].numpy(), v=out[1].numpy(), **{f"p{i}": t.numpy() for i, t in enumerate(out[2:])})
    dist.destroy_process_group()


def test_two_rank_shard_and_reduce_matches_full_grid():
    import oracle as O

    path = os.path.join(tempfile.mkdtemp(), "sum.npz")
    port = 29500 + os.getpid() % 1000
    mp.start_processes(_rank, args=(2, port, path), nprocs=2, start_method="spawn")
    got = np.load(path)
    wl = synthetic.make_workload(1000, 16, 3, seed=4, box_angstrom=6.0, centre_box_angstrom=4.0)
    ao, g1, g2 = O.eval_ao_planes(wl.basis, wl.coords)
    rho = np.einsum("sab,ra,rb->rs", wl.rdm1, ao, ao)
    ehf = synthetic.make_ehf(1000, 2, rho, 2)
    params = synthetic.glorot_params(layer_widths=(32, 32), seed=1)
    e, v, dp = O.xc_energy_and_grads("DM21", wl.rdm1, ao, g1, g2, wl.weights, params=params, ehf=ehf,
                                     want_param_grads=True)
    assert abs(float(got["e"]) - e) <= 1e-12 * abs(e)
    assert np.max(np.abs(got["v"] - v)) <= 1e-12 * np.max(np.abs(v))
    leaves = [dp["params"][k][kk] for k in sorted(dp["params"]) for kk in sorted(dp["params"][k])]
    for i, g in enumerate(leaves):
        assert np.max(np.abs(got[f"p{i}"] - g)) <= 1e-11 * max(np.max(np.abs(g)), 1e-300), i
