"""Host logic of engine.Resident that needs no GPU: the per-network workspace cache."""
import ctypes

import torch

from graddft_gb300 import engine


class _Net:
    def __init__(self, key, nbytes):
        self.key, self.nbytes = key, nbytes
        self.desc = ctypes.c_int(0)


def _resident():
    r = object.__new__(engine.Resident)  # no device buffers: only the cache is exercised
    r.desc = ctypes.c_int(0)
    r.device = torch.device("cpu")
    return r


def test_network_workspaces_cached_per_key():
    """Alternating networks (the DM21 inputs' default network beside a functional's own) keep one zeroed
    workspace each instead of reallocating on every switch; the oldest goes beyond the kept count."""
    r = _resident()
    calls = []
    nets = {}

    def size_fn(desc, net_desc, out):
        net = nets[id(net_desc._obj)]
        calls.append(net.key)
        out._obj.value = net.nbytes
        return 0

    a, b = _Net(("a",), 64), _Net(("b",), 32)
    for n in (a, b):
        nets[id(n.desc)] = n
    wa = r._cached_ws("_nws", a, size_fn)
    wb = r._cached_ws("_nws", b, size_fn)
    for _ in range(3):
        assert r._cached_ws("_nws", a, size_fn) is wa
        assert r._cached_ws("_nws", b, size_fn) is wb
    assert calls == [("a",), ("b",)]
    assert wa.numel() == 64 and int(wa.sum()) == 0 and wb.numel() == 32
    extra = [_Net((f"n{i}",), 8) for i in range(engine.Resident._WS_KEEP)]
    for n in extra:
        nets[id(n.desc)] = n
        r._cached_ws("_nws", n, size_fn)
    assert len(r._nws) == engine.Resident._WS_KEEP and ("a",) not in r._nws


def test_dm21_hf_terms_sum_omegas_in_one_contraction(monkeypatch):
    """dm21_hfgrads_* return the omega sum of the molecule's per-omega HF Fock terms; with the library's
    Molecule they take it as one contraction over both omegas, a Molecule subclass keeps its own method."""
    import numpy as np

    from graddft_gb300 import molecule, neural

    calls = []

    def hf_fock(ao, chi, g, form="fp64"):  # F_s = -1/2 sum_w sum_r ao_ra g_wsr chi_rwsb
        calls.append(chi.shape[1])
        return -0.5 * torch.einsum("rwsb,wsr,ra->sab", chi, g, ao)

    monkeypatch.setattr(engine, "require_cuda", lambda device=None: torch.device("cpu"))
    monkeypatch.setattr(engine, "hf_fock", hf_fock)
    rng = np.random.default_rng(3)
    n_grid, n = 50, 6
    t = lambda a: torch.as_tensor(a, dtype=torch.float64)  # noqa: E731
    mol = molecule.Molecule(grid=molecule.Grid(coords=None, weights=t(rng.random(n_grid))), atom_index=None,
                            nuclear_pos=None, ao=t(rng.standard_normal((n_grid, n))), grad_ao=None, grad_n_ao=None,
                            rdm1=t(rng.standard_normal((2, n, n))), nuclear_repulsion=0.0, h1e=None, vj=None,
                            mo_coeff=None, mo_occ=None, mo_energy=None, omegas=[0.0, 0.4],
                            chi=t(rng.standard_normal((n_grid, 2, 2, n))))
    g = {"hf_density_gradient": t(rng.standard_normal((2, 2, n_grid))),
         "hf_cinput_gradient": t(rng.standard_normal((2, 2, n_grid)))}

    class Fn:
        def hf_density_gradient(self, params, atoms, ehf, clip):
            return g["hf_density_gradient"]

        def hf_cinput_gradient(self, params, atoms, ehf, clip):
            return g["hf_cinput_gradient"]

    for term, method in ((neural.dm21_hfgrads_densities, "HF_density_grad_2_Fock"),
                         (neural.dm21_hfgrads_cinputs, "HF_coefficient_input_grad_2_Fock")):
        calls.clear()
        got = term(Fn(), {}, mol, None, None, None)
        assert calls == [2]  # both omegas in one contraction
        per_omega = getattr(mol, method)(Fn(), {}, (0.0, 0.4), None, None, None)
        assert per_omega.shape == (2, 2, n, n)
        torch.testing.assert_close(got, per_omega.sum(0), rtol=0, atol=1e-12)

    class Custom(molecule.Molecule):
        def HF_density_grad_2_Fock(self, *args, **kwargs):
            return torch.ones((2, 2, n, n), dtype=torch.float64)

    custom = Custom(**{f.name: getattr(mol, f.name) for f in __import__("dataclasses").fields(mol)})
    assert torch.equal(neural.dm21_hfgrads_densities(Fn(), {}, custom, None, None, None),
                       torch.full((2, n, n), 2.0, dtype=torch.float64))
