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
    retired = []
    r._retire_ws = retired.append
    r._cached_ws("_nws", a, size_fn)  # a is now the most recently used: b goes first
    extra = [_Net((f"n{i}",), 8) for i in range(engine.Resident._WS_KEEP - 1)]
    for n in extra:
        nets[id(n.desc)] = n
        r._cached_ws("_nws", n, size_fn)
    assert len(r._nws) == engine.Resident._WS_KEEP and ("b",) not in r._nws and ("a",) in r._nws
    assert retired == [wb]


def test_dropped_workspace_error_word_is_reported(monkeypatch):
    """A bounded wait that expired in a network workspace the cache drops is still reported: the dropped
    workspace's error word is read on the way out and the next status() raises."""
    import pytest

    from graddft_gb300 import _lib

    bad = torch.zeros(16, dtype=torch.uint8)

    class FakeLib:
        def gdft_device_status(self, desc, ws, nbytes, status, stream):
            code = 7 if ws.value == bad.data_ptr() else 0
            status._obj.value = code
            return _lib.GDFT_ERR_DEVICE if code else _lib.GDFT_OK

    monkeypatch.setattr(_lib, "load", lambda *a, **k: FakeLib())
    monkeypatch.setattr(engine, "_stream", lambda device: None)
    r = _resident()
    r.ws = torch.zeros(16, dtype=torch.uint8)
    r._retire_ws(bad)
    with pytest.raises(_lib.GdftError, match="code 7"):
        r.status()
    assert r.status() == 0  # reported once


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


def test_feature_power_columns_host_side():
    """energy_densities=partial(dm21_densities | densities, functional_type=...) resolve to device columns
    on the host: the reference's order (i over u_range, j over w_range; densities() spin-major exchange
    terms, then the zero correlation features), dict ranges, and the reference's ValueError."""
    import functools

    import pytest

    import graddft_gb300 as G
    from graddft_gb300 import _lib
    from graddft_gb300.functional import energy_density_columns as cols

    assert cols(G.dm21_densities) == (_lib.COL_DM21_LDA,)
    assert cols(functools.partial(G.dm21_densities, functional_type="GGA")) == (
        _lib.COL_DM21_LDA, _lib.col_dm21_uw(1, 0))
    assert cols(functools.partial(G.dm21_densities, functional_type="MGGA")) == (
        _lib.COL_DM21_LDA, _lib.col_dm21_uw(0, 1), _lib.col_dm21_uw(1, 0), _lib.col_dm21_uw(1, 1))
    dens = cols(functools.partial(G.densities, functional_type="MGGA"))
    assert len(dens) == 16 and dens[8:] == (_lib.COL_ZERO,) * 8
    assert dens[:4] == (_lib.col_dens_x(0, 0, 0), _lib.col_dens_x(1, 0, 0), _lib.col_dens_x(0, 0, 1),
                        _lib.col_dens_x(1, 0, 1))
    d = {"u_range": range(0, 2), "w_range": range(0, 2)}
    assert cols(functools.partial(G.dm21_densities, functional_type=d)) == cols(
        functools.partial(G.dm21_densities, functional_type="MGGA"))
    with pytest.raises(ValueError):
        cols(functools.partial(G.dm21_densities, functional_type="XGGA"))
    with pytest.raises(NotImplementedError):  # 2 * 3 * 3 * 2 columns exceed the device functional
        G.densities(None, {"u_range": range(0, 3), "w_range": range(0, 3)})
    with pytest.raises(NotImplementedError):
        cols(functools.partial(G.dm21_densities, functional_type="GGA", clip_cte=1e-20))
    # the codes the C ABI documents (GDFT_COL_DM21_UW / GDFT_COL_DENS_X)
    assert _lib.col_dm21_uw(1, 1) == 0x111 and _lib.col_dens_x(1, 1, 0) == 0x310


def test_dlpack_producer_is_accepted_on_the_host():
    """as_device_f64 takes an object that offers only __dlpack__ / __dlpack_device__ (a jax.Array's view
    of the protocol), here wrapping a CPU tensor and a numpy array."""
    import numpy as np

    class DLPackOnly:
        def __init__(self, a):
            self._a = a

        def __dlpack__(self, *args, **kwargs):
            return self._a.__dlpack__(*args, **kwargs)

        def __dlpack_device__(self):
            return self._a.__dlpack_device__()

    a = np.arange(12, dtype=np.float32).reshape(3, 4)
    for src in (torch.as_tensor(a), a):
        got = engine.as_device_f64(DLPackOnly(src), "cpu")
        assert got.dtype == torch.float64 and got.is_contiguous()
        assert torch.equal(got, torch.as_tensor(a, dtype=torch.float64))


def test_chunk_autotuner_times_once_and_caches(monkeypatch, tmp_path):
    """The autotuner keeps the smallest chunk within the tolerance of the fastest, skips sizes over the memory
    budget or the grid, and answers from its on-disk cache afterwards."""
    from graddft_gb300 import autotune

    monkeypatch.setenv("GDFT_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    ms = {1 << 14: 10.0, 1 << 15: 8.0, 1 << 16: 7.9, 1 << 17: 7.7, 1 << 18: 7.6}
    timed = []
    monkeypatch.setattr(autotune, "time_call", lambda fn, device, reps=2: (fn(), ms.get(timed[-1], 5.0))[1])
    run = lambda c: timed.append(c)  # noqa: E731
    ws = lambda c: c * 1000  # noqa: E731
    got = autotune.choose("k", run, ws, n_grid=1 << 20, device=None, budget_bytes=(1 << 17) * 1000, tol=0.03)
    assert got == 1 << 16 and sorted(set(timed)) == [1 << 14, 1 << 15, 1 << 16, 1 << 17]
    timed.clear()
    assert autotune.choose("k", run, ws, n_grid=1 << 20, device=None, budget_bytes=1) == 1 << 16 and not timed
    # sizes above the grid collapse to the grid rounded up to 256
    timed.clear()
    assert autotune.choose("small", run, ws, n_grid=5000, device=None, budget_bytes=1 << 40) == 5120
    assert set(timed) == {5120}


def test_longest_first_schedule():
    from graddft_gb300.batch import schedule_longest_first

    q = schedule_longest_first([5, 1, 3, 3, 2, 8], 2)
    assert q == [[5, 3], [0, 2, 4, 1]]
    assert schedule_longest_first([1.0], 3) == [[0], [], []]
    costs = [float(c) for c in range(1, 40)]
    loads = [sum(costs[i] for i in qq) for qq in schedule_longest_first(costs, 4)]
    assert max(loads) - min(loads) <= max(costs)
