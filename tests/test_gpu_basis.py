"""GPU parity of the contracted-shell AO evaluator against the oracle.

gdft_eval_ao stands in for numint.eval_ao (interface/pyscf.py:849-852) plus the
diagonal of ao_grads(order=2) (interface/pyscf.py:677-705);
gdft_molecule_eval_shells fills the resident tables of both arithmetic forms
from the same shells.  Oracle: oracle/shells.py (its own angular rows from
SciPy's harmonics, its own derivative algebra).  Bar: FP64, 1e-12 relative to
the largest entry of each output.
"""
import math

import numpy as np
import pytest
import torch

import oracle as O
from oracle import shells as OS
from graddft_gb300 import synthetic

pytestmark = pytest.mark.gpu

RTOL = 1e-12


@pytest.fixture(scope="module")
def G(built_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import graddft_gb300 as G

    return G


def _close(a, b, rtol=RTOL, what=""):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    b = np.asarray(b)
    assert a.shape == b.shape, (what, a.shape, b.shape)
    scale = max(np.max(np.abs(b)), 1e-300)
    err = np.max(np.abs(a - b))
    assert err <= rtol * scale, f"{what}: max abs err {err:.3e} vs scale {scale:.3e}"


def _random_basis(B, seed, max_l, cart=False, n_copies=2, spread=2.5):
    g = np.random.default_rng(seed)
    shells = []
    for _ in range(n_copies):
        for l in range(max_l + 1):
            nprim = int(g.integers(1, 6))
            nctr = int(g.integers(1, 3))
            e = np.sort(np.exp(g.uniform(math.log(0.1), math.log(40.0), nprim)))[::-1]
            c = B.normalized_contraction(l, e, g.uniform(-0.2, 1.0, (nprim, nctr)))
            shells.append(B.Shell(g.uniform(-spread, spread, 3), l, e, c))
    g.shuffle(shells)
    return B.ShellBasis(shells, cart=cart)


def _spec(basis):
    return [(s.centre, s.l, s.exps, s.coefs, None if s.rows is None else basis.rows_for(s)) for s in basis.shells]


@pytest.mark.parametrize("cart,max_l", [(False, 6), (True, 4)])
def test_eval_ao_vs_oracle(G, cart, max_l):
    from graddft_gb300 import basis as B

    basis = _random_basis(B, 11 + max_l, max_l, cart)
    coords = np.random.default_rng(12).uniform(-4.0, 4.0, (3001, 3))
    ao, g1, g2 = B.eval_ao(basis, coords, deriv=2)
    r_ao, r_g1, r_g2 = OS.eval_shells(_spec(basis), coords, cart=cart)
    assert ao.shape == (3001, basis.n_ao)
    _close(ao, r_ao, what="ao")
    _close(g1, r_g1, what="grad_ao")
    _close(g2, r_g2, what="grad2_ao")
    # lower derivative orders return the same values
    ao0 = B.eval_ao(basis, coords, deriv=0)
    ao1, g11 = B.eval_ao(basis, coords, deriv=1)
    assert torch.equal(ao0, ao) and torch.equal(ao1, ao) and torch.equal(g11, g1)


def test_synthetic_basis_through_shells(G):
    from graddft_gb300 import basis as B

    wl = synthetic.make_workload(2051, 70, 8, seed=13, box_angstrom=7.0, centre_box_angstrom=4.0)
    sb = B.ShellBasis.from_synthetic(wl.basis)
    got = B.eval_ao(sb, wl.coords, deriv=2)
    ref = O.eval_ao_planes(wl.basis, wl.coords)
    for a, b, what in zip(got, ref, ("ao", "grad_ao", "grad2_ao")):
        _close(a, b, what=what)


@pytest.mark.parametrize("precision", ["fp64", "tf32x3"])
def test_resident_from_shells_matches_tables(G, precision):
    """The fused path (shells -> resident tables) gives the same E_xc and V_xc as loading eval_ao's tables."""
    from graddft_gb300 import basis as B

    basis = _random_basis(B, 21, 3, n_copies=6, spread=3.0)
    n = basis.n_ao
    g = np.random.default_rng(22)
    coords = g.uniform(-5.0, 5.0, (4099, 3))
    w = g.lognormal(-3.0, 0.5, 4099)
    rdm1 = synthetic.make_rdm1(n, max(2, n // 4), seed=23)
    ao, g1, g2 = B.eval_ao(basis, coords, deriv=2)
    r_tab = G.engine.Resident.from_tables(ao, g1, g2, w, precision)
    r_sh = G.engine.Resident.from_shells(basis, coords, w, precision)
    if precision == "fp64":
        assert torch.equal(r_tab.ao_planes(), r_sh.ao_planes())
    from graddft_gb300 import _lib, engine

    for cols in ([_lib.COL_B88], [_lib.COL_LYP, _lib.COL_VWN]):
        fn = engine.make_functional(cols, [1.0] * len(cols))
        e1, v1 = r_sh.xc_energy_and_grads(rdm1, fn)
        e2, v2 = r_tab.xc_energy_and_grads(rdm1, fn)
        assert float(e1) == float(e2)
        assert torch.equal(v1, v2)
    d1, d2 = r_sh.density(rdm1), r_tab.density(rdm1)
    for k in d1:
        assert torch.equal(d1[k], d2[k]), k


def test_molecule_from_basis_vs_oracle_tables(G):
    """B3LYP energy and Fock matrix from device-evaluated shells against the oracle's tables."""
    from graddft_gb300 import basis as B

    basis = _random_basis(B, 31, 2, n_copies=3, spread=2.0)
    n = basis.n_ao
    g = np.random.default_rng(32)
    coords = g.uniform(-4.0, 4.0, (2500, 3))
    w = g.lognormal(-3.0, 0.5, 2500)
    rdm1 = synthetic.make_rdm1(n, max(2, n // 3), seed=33)
    h1e = np.eye(n) * 0.1
    eri = np.zeros((n, n, n, n))
    mol = B.molecule_from_basis(basis, coords, w, rdm1, h1e=torch.as_tensor(h1e, device="cuda"),
                                rep_tensor=torch.as_tensor(eri, device="cuda"), nuclear_repulsion=1.0)
    ao, g1, g2 = OS.eval_shells(_spec(basis), coords)
    t = lambda x: torch.as_tensor(x, dtype=torch.float64, device="cuda")  # noqa: E731
    ref = G.Molecule(grid=G.Grid(coords=None, weights=t(w)), atom_index=None, nuclear_pos=None, ao=t(ao),
                     grad_ao=t(g1), grad_n_ao={2: t(g2)}, rdm1=t(rdm1), nuclear_repulsion=1.0, h1e=t(h1e),
                     vj=None, mo_coeff=None, mo_occ=None, mo_energy=None, rep_tensor=t(eri))
    E1, F1 = G.energy_predictor(G.LSDA)({"params": {}}, mol)
    E2, F2 = G.energy_predictor(G.LSDA)({"params": {}}, ref)
    assert abs(float(E1) - float(E2)) <= 1e-11 * abs(float(E2))
    _close(F1, F2.cpu().numpy(), rtol=1e-11, what="Fock")


def test_errors(G):
    from graddft_gb300 import basis as B

    basis = _random_basis(B, 41, 1, n_copies=1)
    with pytest.raises(ValueError):
        B.eval_ao(basis, np.zeros((5, 2)))
    with pytest.raises(ValueError):
        B.eval_ao(basis, np.zeros((5, 3)), deriv=3)
    r = G.engine.Resident(16, basis.n_ao + 1, "fp64")
    desc, _keep = basis.device_desc(r.device)
    import ctypes

    c = torch.zeros((16, 3), dtype=torch.float64, device="cuda")
    w = torch.ones(16, dtype=torch.float64, device="cuda")
    with pytest.raises(ValueError):  # n_ao mismatch
        G._lib.check(G._lib.load().gdft_molecule_eval_shells(ctypes.byref(r.desc), ctypes.byref(desc),
                                                             ctypes.c_void_p(c.data_ptr()),
                                                             ctypes.c_void_p(w.data_ptr()), None))
    with pytest.raises(ValueError):  # no basis
        G._lib.check(G._lib.load().gdft_eval_ao(None, ctypes.c_void_p(c.data_ptr()), 16, 0,
                                                ctypes.c_void_p(c.data_ptr()), None, None, None))
