"""GPU parity of the exact-exchange (HF) terms computed from a chi tensor.

HF_energy_density (molecule.py:507-541), the HF Fock terms of B3LYP
(HF_density_grad_2_Fock, molecule.py:545-613, summed over omega by
b3lyp_hfgrads) and of DM21 (dm21_hfgrads_densities / dm21_hfgrads_cinputs,
functional.py:677-757), and energy_predictor with those terms
(train.py:124-218) against fixtures made by running the reference's own source
(tests/golden/make_golden.py), and the general-omega Fock contraction against
the oracle.  FP64 form: the bar is 1e-11 relative to the largest entry; the
mixed form's exchange contractions (three-slice tensor-core GEMM): 2e-8.
"""
import numpy as np
import pytest
import torch

import oracle as O
from graddft_gb300 import synthetic

pytestmark = pytest.mark.gpu

RTOL = 1e-11


def _close(a, b, rtol=RTOL, what=""):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    b = np.asarray(b)
    assert a.shape == b.shape, (what, a.shape, b.shape)
    scale = max(np.max(np.abs(b)), 1e-300)
    err = np.max(np.abs(a - b))
    assert err <= rtol * scale, f"{what}: max abs err {err:.3e} vs scale {scale:.3e}"


@pytest.fixture(scope="module")
def G(built_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import graddft_gb300 as G

    return G


def _t(x):
    return torch.as_tensor(np.asarray(x), dtype=torch.float64, device="cuda")


def _molecule(G, g, precision="fp64"):
    grid = G.Grid(coords=None, weights=_t(g["weights"]))
    return G.Molecule(grid=grid, atom_index=None, nuclear_pos=None, ao=_t(g["ao"]), grad_ao=_t(g["grad_ao"]),
                      grad_n_ao={2: _t(g["grad2_ao"])}, rdm1=_t(g["rdm1"]), nuclear_repulsion=1.25, h1e=_t(g["h1e"]),
                      vj=None, mo_coeff=None, mo_occ=None, mo_energy=None, rep_tensor=_t(g["eri"]),
                      omegas=[float(o) for o in g["omegas"]], chi=_t(g["chi"]), precision=precision)


def test_hf_energy_density(G, golden):
    g = golden("hf")
    mol = _molecule(G, g)
    _close(mol.HF_energy_density([0.0, 0.4]), g["ehf"], what="ehf")
    _close(mol.HF_energy_density([0.0]), g["ehf_w0"], what="ehf w0")
    # omega order follows the request, as in select_HF_omegas
    _close(mol.HF_energy_density([0.4, 0.0]), g["ehf"][::-1], what="ehf reversed")


def test_b3lyp_hf_fock_term(G, golden):
    g = golden("hf")
    mol = _molecule(G, g)
    ehf0 = mol.HF_energy_density([0.0])
    v = G.popular_functionals.b3lyp_hfgrads(G.B3LYP, {"params": {}}, mol, ehf0, None, None)
    _close(v, g["b3lyp_hfgrads"], what="b3lyp_hfgrads")


@pytest.mark.parametrize("precision", ["fp64", "tf32x3"])
def test_b3lyp_predict_with_chi(G, golden, precision):
    g = golden("hf")
    mol = _molecule(G, g, precision)
    E, F = G.energy_predictor(G.B3LYP)({"params": {}}, mol)
    # The mixed form's E_xc and V_xc carry its ~1e-7 relative error; its exchange terms about 1e-9.
    rtol = RTOL if precision == "fp64" else 2e-6
    assert abs(float(E) - float(g["predict_E_B3LYP"])) <= rtol * abs(float(g["predict_E_B3LYP"]))
    _close(F, g["predict_F_B3LYP"], rtol=rtol, what="F")


def test_hf_fock_general_omegas_vs_oracle(G):
    """Two omegas, omega- and spin-dependent g, ragged sizes."""
    n_grid, n_ao = 4099, 37
    wl = synthetic.make_workload(n_grid, n_ao, 5, seed=21, box_angstrom=7.0, centre_box_angstrom=4.0)
    ao, _, _ = O.eval_ao_planes(wl.basis, wl.coords)
    chi = synthetic.make_chi(ao, wl.rdm1, n_omega=2, seed=22)
    rng = np.random.default_rng(23)
    gw = rng.standard_normal((2, 2, n_grid)) * 1e-3
    got = G.engine.hf_fock(_t(ao), _t(chi), _t(gw))
    ref = (-0.5 * np.einsum("rwsb,wsr,ra->sab", chi, gw, ao))
    _close(got, ref, what="hf_fock")
    e = G.engine.hf_energy_density(_t(ao), _t(wl.rdm1), _t(chi))
    _close(e, O.hf_energy_density(wl.rdm1, ao, chi).numpy(), what="ehf")


MIXED_RTOL = 2e-8  # three-slice operands: about 2^-31 of each row's largest entry per element


@pytest.mark.parametrize("n_grid,n_ao,n_omega", [(4099, 37, 2), (1000, 130, 3), (31, 5, 1)])
def test_hf_mixed_form_vs_oracle(G, n_grid, n_ao, n_omega):
    """The tensor-core (TF32x3) exact-exchange contractions on ragged sizes: partial point tiles and
    K chunks, both spins in one GEMM with a spin boundary inside a column tile (n_ao = 130), a single
    partial tile (31 points x 5 orbitals); numpy emulation of the six-product form: 4e-10 (F), 1e-9 (ehf)."""
    wl = synthetic.make_workload(n_grid, n_ao, max(1, min(5, n_ao // 2)), seed=21, box_angstrom=7.0,
                                 centre_box_angstrom=4.0)
    ao, _, _ = O.eval_ao_planes(wl.basis, wl.coords)
    chi = synthetic.make_chi(ao, wl.rdm1, n_omega=n_omega, seed=22)
    rng = np.random.default_rng(23)
    gw = rng.standard_normal((n_omega, 2, n_grid)) * 1e-3
    ref_f = -0.5 * np.einsum("rwsb,wsr,ra->sab", chi, gw, ao)
    ref_e = O.hf_energy_density(wl.rdm1, ao, chi).numpy()
    got_f = G.engine.hf_fock(_t(ao), _t(chi), _t(gw), form="tf32x3")
    _close(got_f, ref_f, rtol=MIXED_RTOL, what="hf_fock (mixed)")
    got_e = G.engine.hf_energy_density(_t(ao), _t(wl.rdm1), _t(chi), form="tf32x3")
    _close(got_e, ref_e, rtol=MIXED_RTOL, what="ehf (mixed)")
    # the FP64 form of the same call stays at FP64 rounding
    _close(G.engine.hf_fock(_t(ao), _t(chi), _t(gw), form="fp64"), ref_f, what="hf_fock (fp64)")


def test_hf_mixed_form_golden(G, golden):
    """ehf and the B3LYP HF Fock term in the mixed form against the reference's own outputs."""
    g = golden("hf")
    mol = _molecule(G, g, precision="tf32x3")
    _close(mol.HF_energy_density([0.0, 0.4]), g["ehf"], rtol=MIXED_RTOL, what="ehf (mixed)")
    ehf0 = mol.HF_energy_density([0.0])
    v = G.popular_functionals.b3lyp_hfgrads(G.B3LYP, {"params": {}}, mol, ehf0, None, None)
    _close(v, g["b3lyp_hfgrads"], rtol=1e-6, what="b3lyp_hfgrads (mixed densities and exchange)")


def test_hf_errors(G, golden):
    g = golden("hf")
    mol = _molecule(G, g)
    with pytest.raises(ValueError):
        mol.HF_energy_density([0.2])  # omega not in molecule.omegas (molecule.py:176-180)
    with pytest.raises(ValueError):
        G.engine.hf_energy_density(_t(g["ao"]), _t(g["rdm1"]), _t(g["chi"])[:, :, :, :5])
    no_chi = mol.replace(chi=None)
    with pytest.raises(ValueError):
        no_chi.HF_energy_density([0.0])
    with pytest.raises(ValueError):
        G.engine.hf_energy_density(_t(g["ao"]), _t(g["rdm1"]), _t(g["chi"]), form="bf16")


def test_dm21_hf_terms(G, golden):
    g = golden("hf")
    mol = _molecule(G, g)
    dm21 = G.DM21()
    params = synthetic.glorot_params(seed=int(g["theta_seed"]))
    ehf = mol.HF_energy_density([0.0, 0.4])
    fd = G.neural.dm21_hfgrads_densities(dm21, params, mol, ehf, None, None)
    fc = G.neural.dm21_hfgrads_cinputs(dm21, params, mol, ehf, None, None)
    _close(fd, g["dm21_hfgrads_densities"], what="HF term through the densities")
    _close(fc, g["dm21_hfgrads_cinputs"], what="HF term through the inputs")


def test_dm21_predict_with_chi(G, golden):
    g = golden("hf")
    mol = _molecule(G, g)
    params = synthetic.glorot_params(seed=int(g["theta_seed"]))
    E, F = G.energy_predictor(G.DM21())(params, mol)
    assert abs(float(E) - float(g["predict_E_DM21"])) <= RTOL * abs(float(g["predict_E_DM21"]))
    _close(F, g["predict_F_DM21"], what="F")


@pytest.mark.parametrize("mol_form", ["fp64", "tf32x3"])
def test_dm21_hf_terms_and_predict_mixed_network(G, golden, mol_form):
    """The same with the tensor-core (TF32x3) network: E to 1e-6 relative, the HF terms and F to 2e-5 of
    their largest entries (the network's FP32 activations), with the molecule's densities, V_xc and
    exchange contractions in either form."""
    g = golden("hf")
    mol = _molecule(G, g, mol_form)
    params = synthetic.glorot_params(seed=int(g["theta_seed"]))
    dm21 = G.DM21(precision="tf32x3")
    ehf = mol.HF_energy_density([0.0, 0.4])
    fd = G.neural.dm21_hfgrads_densities(dm21, params, mol, ehf, None, None)
    fc = G.neural.dm21_hfgrads_cinputs(dm21, params, mol, ehf, None, None)
    _close(fd, g["dm21_hfgrads_densities"], rtol=2e-5, what="HF term through the densities (mixed network)")
    _close(fc, g["dm21_hfgrads_cinputs"], rtol=2e-5, what="HF term through the inputs (mixed network)")
    E, F = G.energy_predictor(dm21)(params, mol)
    assert abs(float(E) - float(g["predict_E_DM21"])) <= 1e-6 * abs(float(g["predict_E_DM21"]))
    _close(F, g["predict_F_DM21"], rtol=2e-5, what="F (mixed network)")


@pytest.mark.parametrize("precision", ["fp64", "tf32x3"])
def test_b3lyp_n43_config1_stand_in(G, golden, precision):
    """Config 1's stand-in (n_ao 43, unrestricted B3LYP on a fixed D, HF column from chi): E_xc, V_xc and
    the explicit HF Fock term against the reference's own outputs (inputs regenerated from seeds)."""
    from oracle.cases import b3lyp43_inputs

    g = golden("b3lyp43")
    wl, ao, g1, g2, chi, omegas = b3lyp43_inputs()
    mol = G.Molecule(grid=G.Grid(coords=None, weights=_t(wl.weights)), atom_index=None, nuclear_pos=None,
                     ao=_t(ao), grad_ao=_t(g1), grad_n_ao={2: _t(g2)}, rdm1=_t(wl.rdm1), nuclear_repulsion=0.0,
                     h1e=None, vj=None, mo_coeff=None, mo_occ=None, mo_energy=None, rep_tensor=None,
                     omegas=[float(o) for o in omegas], chi=_t(chi), precision=precision)
    exc, vxc = G.B3LYP.xc_energy_and_grads({"params": {}}, mol)
    ehf0 = mol.HF_energy_density([0.0])
    vhf = G.popular_functionals.b3lyp_hfgrads(G.B3LYP, {"params": {}}, mol, ehf0, None, None)
    # Mixed form: E_xc and V_xc at the mixed tolerances; the exchange terms' three-slice GEMMs at 2e-8.
    rtol_e, rtol_v, rtol_hf = (RTOL, RTOL, RTOL) if precision == "fp64" else (5e-7, 2e-6, 2e-8)
    ref = float(g["exc"])
    assert abs(float(exc) - ref) <= rtol_e * abs(ref), (float(exc), ref)
    _close(vxc, g["vxc"], rtol=rtol_v, what="V_xc")
    _close(ehf0, g["ehf"], rtol=rtol_hf, what="ehf")
    _close(vhf, g["b3lyp_hfgrads"], rtol=max(rtol_hf, 2e-6 if precision != "fp64" else RTOL), what="HF Fock term")
