"""Batched molecules (one network pass over all grid points, per-molecule energies
and loss cotangents on the device) against one-at-a-time evaluation, and CUDA-graph replay."""
import numpy as np
import pytest
import torch

import oracle as O
from graddft_gb300 import synthetic

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G(built_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import graddft_gb300 as G

    return G


def _t(x):
    return torch.as_tensor(np.asarray(x), dtype=torch.float64, device="cuda")


def _molecules(G, shapes, precision="tf32x3"):
    mols = []
    for i, (n_ao, n_grid) in enumerate(shapes):
        wl = synthetic.make_workload(n_grid, n_ao, max(1, n_ao // 8), seed=80 + i, box_angstrom=8.0,
                                     centre_box_angstrom=5.0)
        ao, g1, g2 = O.eval_ao_planes(wl.basis, wl.coords)
        rho = np.einsum("sab,ra,rb->rs", wl.rdm1, ao, ao)
        ehf = synthetic.make_ehf(n_grid, 90 + i, rho, 2)
        mols.append(G.Molecule(grid=G.Grid(coords=None, weights=_t(wl.weights)), atom_index=None, nuclear_pos=None,
                               ao=_t(ao), grad_ao=_t(g1), grad_n_ao={2: _t(g2)}, rdm1=_t(wl.rdm1),
                               nuclear_repulsion=0.0, h1e=None, vj=None, mo_coeff=None, mo_occ=None, mo_energy=None,
                               ehf=_t(ehf), precision=precision))
    return mols


def _dm21(G):
    hf = lambda atoms, *_, **__: atoms.ehf  # noqa: E731
    return G.DM21(densitygrads=None, coefficient_input_grads=None, nograd_densities=hf, nograd_coefficient_inputs=hf,
                  precision="tf32x3")


SHAPES = [(20, 1000), (40, 2048), (64, 3000), (130, 4096)]


def test_batch_matches_one_at_a_time(G):
    from graddft_gb300.batch import NeuralBatch

    mols = _molecules(G, SHAPES)
    f = _dm21(G)
    params = f.init(11)
    seq = [f.xc_energy_and_grads_params(params, m) for m in mols]
    e_ref = np.array([float(s[0]) for s in seq]) + 0.01 * np.arange(len(mols))
    b = NeuralBatch(mols, f)
    loss, energies, vxcs, dp = b.step(params, eref=e_ref)
    assert b.status() == 0
    for m, (e, v, _) in enumerate(seq):
        assert abs(float(energies[m]) - float(e)) <= 1e-12 * abs(float(e)) + 1e-15, (m, float(energies[m]), float(e))
        g = 2.0 * (float(e) - e_ref[m])
        err = float((vxcs[m] - g * v).abs().max()) / max(float((g * v).abs().max()), 1e-300)
        # The batch seeds the FP32 backward with (g dy) rounded once, the reference g (dy rounded): ~1e-7.
        assert err <= 1e-6, (m, err)
    want = sum(2.0 * (float(s[0]) - e_ref[m]) * b.net.flatten(s[2], b.device) for m, s in enumerate(seq))
    assert abs(float(loss) - float(((np.array([float(s[0]) for s in seq]) - e_ref) ** 2).sum())) <= 1e-12
    rel = float((dp - want).abs().max()) / float(want.abs().max())
    assert rel <= 1e-6, rel


def test_batch_graph_replay(G):
    from graddft_gb300.batch import NeuralBatch

    mols = _molecules(G, SHAPES[:3])
    f = _dm21(G)
    b = NeuralBatch(mols, f)
    b.set_inputs(params=f.init(3))
    b.capture()
    rng = np.random.default_rng(4)
    new_d = [m._rdm1() * (1.0 + 0.01 * rng.standard_normal()) for m in mols]
    b.set_inputs(rdm1s=new_d)
    loss, e_graph, v_graph, d_graph = [x.clone() if isinstance(x, torch.Tensor) else [t.clone() for t in x]
                                       for x in b.replay()]
    loss2, e_eager, v_eager, d_eager = b.step()
    assert torch.equal(e_graph, e_eager)
    assert all(torch.equal(a, c) for a, c in zip(v_graph, v_eager))
    assert torch.equal(d_graph, d_eager)
    assert b.status() == 0


def test_batch_status_reports_a_recorded_expiry(G):
    """The batch's persistent error word: a code recorded there (planted from the host, as an expired
    bounded wait would leave it) is reported once by status() and then cleared."""
    from graddft_gb300 import _lib
    from graddft_gb300.batch import NeuralBatch

    mols = _molecules(G, SHAPES[:2])
    f = _dm21(G)
    b = NeuralBatch(mols, f)
    b.step(f.init(5))
    assert b.status() == 0
    b.ws[:4].copy_(torch.tensor([46, 0, 0, 0], dtype=torch.uint8))
    with pytest.raises(_lib.GdftError):
        b.status()
    assert b.status() == 0
    # The shared molecule region is the largest molecule's, not the sum over the batch.
    import ctypes

    one = []
    for r in b.residents:
        nb = ctypes.c_size_t()
        _lib.check(_lib.load().gdft_neural_batch_workspace_bytes(1, ctypes.byref(r.desc), ctypes.byref(b.net.desc),
                                                                 ctypes.byref(nb)))
        one.append(nb.value)
    assert b.ws.numel() < sum(one)
