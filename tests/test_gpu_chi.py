"""GPU parity of the nu integrals and the chi tensor.

gdft_nu_integrals stands in for PySCF's int1e_grids as _evaluate_nu calls it
(external/_hf_density.py:17-120); gdft_chi for generate_chi_tensor
(interface/pyscf.py:1067-1126).  Checked against the oracle (oracle/nu.py,
itself pinned by quadrature and closed forms) and against the fixture of the
reference's generate_chi_tensor (tests/golden/ref_chi.npz).  FP64: 1e-12
relative to the largest entry.
"""
import math

import numpy as np
import pytest
import torch

from oracle import nu as ONU
from oracle import shells as OS

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


def _fixture_basis(G, g):
    from graddft_gb300 import basis as B

    shells = [B.Shell(g[f"shell{i}/centre"], int(g[f"shell{i}/l"]), g[f"shell{i}/exps"], g[f"shell{i}/coefs"])
              for i in range(int(g["n_shell"]))]
    spec = [(s.centre, s.l, s.exps, s.coefs, None) for s in shells]
    return B.ShellBasis(shells), spec


@pytest.mark.parametrize("omega", [0.0, 0.4, 1.5])
def test_nu_integrals_vs_oracle(G, golden, omega):
    g = golden("chi")
    basis, spec = _fixture_basis(G, g)
    pts = g["coords"][:70]
    got = G.chi.nu_integrals(basis, pts, omega)
    _close(got, ONU.nu_integrals(spec, pts, omega), what=f"nu omega={omega}")
    assert torch.equal(got, got.transpose(1, 2))


@pytest.mark.parametrize("chunk", [64, 37, 1000])
def test_chi_vs_reference_fixture(G, golden, chunk):
    g = golden("chi")
    basis, _ = _fixture_basis(G, g)
    chi = G.chi.generate_chi_tensor(g["rdm1"], g["ao"], g["coords"], basis, list(g["omegas"]), chunk_size=chunk)
    _close(chi, g["chi"], what=f"chi chunk={chunk}")


@pytest.mark.parametrize("cart", [False, True])
def test_random_basis_vs_oracle(G, cart):
    from graddft_gb300 import basis as B

    rng = np.random.default_rng(71 + cart)
    shells = []
    for _ in range(4):
        c = rng.uniform(-2.0, 2.0, 3)
        for l in (0, 1, 2, 3):
            nprim = int(rng.integers(1, 4))
            nctr = int(rng.integers(1, 3))
            e = np.sort(np.exp(rng.uniform(math.log(0.1), math.log(30.0), nprim)))[::-1]
            shells.append(B.Shell(c, l, e, B.normalized_contraction(l, e, rng.uniform(0.1, 1.0, (nprim, nctr)))))
    rng.shuffle(shells)
    basis = B.ShellBasis(shells, cart=cart)
    spec = [(s.centre, s.l, s.exps, s.coefs, None) for s in shells]
    pts = rng.uniform(-4.0, 4.0, (45, 3))
    for omega in (0.0, 0.3):
        _close(G.chi.nu_integrals(basis, pts, omega), ONU.nu_integrals(spec, pts, omega, cart=cart),
               what=f"nu cart={cart} omega={omega}")


def test_chi_many_omegas(G, golden):
    """More omegas than one library call takes: split and concatenated in omega order."""
    g = golden("chi")
    basis, spec = _fixture_basis(G, g)
    sl = slice(0, 40)
    omegas = [0.0, 0.1, 0.2, 0.3, 0.4, 0.5, 0.6, 0.7, 0.8, 1.0]
    chi = G.chi.generate_chi_tensor(g["rdm1"], g["ao"][sl], g["coords"][sl], basis, omegas, chunk_size=16)
    assert chi.shape == (40, 10, 2, 30)
    ref = ONU.generate_chi(g["rdm1"], g["ao"][sl], [ONU.nu_integrals(spec, g["coords"][sl], w) for w in omegas])
    _close(chi, ref, what="chi 10 omegas")


def test_chi_feeds_hf_energy_density(G, golden):
    """chi generated on the device gives the oracle's HF energy density (molecule.py:507-541)."""
    import oracle as O

    g = golden("chi")
    basis, _ = _fixture_basis(G, g)
    chi = G.chi.generate_chi_tensor(g["rdm1"], g["ao"], g["coords"], basis, [0.0, 0.4])
    t = lambda x: torch.as_tensor(np.asarray(x), dtype=torch.float64, device="cuda")  # noqa: E731
    ehf = G.engine.hf_energy_density(t(g["ao"]), t(g["rdm1"]), chi)
    ref = O.hf_energy_density(g["rdm1"], g["ao"], g["chi"]).numpy()
    _close(ehf, ref, what="ehf")


def test_errors(G):
    from graddft_gb300 import basis as B

    g_shell = B.ShellBasis([B.Shell(np.zeros(3), 4, np.array([1.0]), np.array([[1.0]]))])
    with pytest.raises(NotImplementedError):
        G.chi.nu_integrals(g_shell, np.zeros((4, 3)), 0.0)
    s_shell = B.ShellBasis([B.Shell(np.zeros(3), 0, np.array([1.0]), np.array([[1.0]]))])
    with pytest.raises(ValueError):
        G.chi.nu_integrals(s_shell, np.zeros((4, 3)), -0.1)
    with pytest.raises(ValueError):
        G.chi.generate_chi_tensor(np.zeros((2, 1, 1)), np.zeros((4, 1)), np.zeros((4, 3)), s_shell, [0.0, -1.0])
    assert G.chi.generate_chi_tensor(np.zeros((2, 1, 1)), np.zeros((4, 1)), np.zeros((4, 3)), s_shell, []).numel() == 0
    with pytest.raises(ValueError):  # rdm1 shape
        G.chi.generate_chi_tensor(np.zeros((1, 1, 1)), np.zeros((4, 1)), np.zeros((4, 3)), s_shell, [0.0])
