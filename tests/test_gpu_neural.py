"""GPU parity of the DM21-style neural functional (FP64 form) through the C ABI.

Checked against the reference's own outputs (tests/golden/ref_dm21.npz: E_xc,
V_xc, coefficient inputs, densities, coefficients and dE/dtheta subsets from
jax.grad), against the oracle at a larger size, against central finite
differences in theta and in the density matrix, and through the
torch.autograd.Function that carries the hand-written adjoint.
"""
import numpy as np
import pytest
import torch

import oracle as O
from graddft_gb300 import synthetic

pytestmark = pytest.mark.gpu

RTOL = 1e-10  # FP64 form: differs from the reference only in summation order


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


def _molecule(G, ao, g1, g2, w, rdm1, ehf, precision="fp64"):
    return G.Molecule(grid=G.Grid(coords=None, weights=_t(w)), atom_index=None, nuclear_pos=None, ao=_t(ao),
                      grad_ao=_t(g1), grad_n_ao={2: _t(g2)}, rdm1=_t(rdm1), nuclear_repulsion=0.0, h1e=None,
                      vj=None, mo_coeff=None, mo_occ=None, mo_energy=None, ehf=_t(ehf), precision=precision)


def _dm21(G):
    hf = lambda atoms, *_, **__: atoms.ehf  # noqa: E731  (stop-gradient supplied HF densities)
    return G.DM21(densitygrads=None, coefficient_input_grads=None, nograd_densities=hf, nograd_coefficient_inputs=hf)


def _params(seed=7):
    p = synthetic.glorot_params(seed=seed)
    return {"params": {k: {kk: torch.as_tensor(v) for kk, v in d.items()} for k, d in p["params"].items()}}


@pytest.fixture(scope="module")
def ref(golden):
    return golden("dm21")


def test_inputs_densities_coefficients(G, ref):
    mol = _molecule(G, ref["ao"], ref["grad_ao"], ref["grad2_ao"], ref["weights"], ref["rdm1"], ref["ehf"])
    f = _dm21(G)
    cin = f.compute_coefficient_inputs(mol)
    for k in range(11):
        _close(cin[:, k], ref["cinputs"][:, k], what=f"cinput {k}")
    _close(f.compute_densities(mol), ref["densities"], what="densities")
    c = f.apply(_params(int(ref["theta_seed"])), cin)
    _close(c, ref["coefficients"], what="coefficients")


def test_energy_vxc_dtheta_vs_reference(G, ref):
    mol = _molecule(G, ref["ao"], ref["grad_ao"], ref["grad2_ao"], ref["weights"], ref["rdm1"], ref["ehf"])
    f = _dm21(G)
    e, v, dp = f.xc_energy_and_grads_params(_params(int(ref["theta_seed"])), mol)
    assert abs(float(e) - float(ref["exc"])) <= RTOL * abs(float(ref["exc"])), (float(e), float(ref["exc"]))
    _close(v, ref["vxc"], what="V_xc")
    n_checked = 0
    for key in ref.files:
        if not key.startswith("dtheta/") or key.endswith("/idx"):
            continue
        _, mod, leaf = key.split("/")
        got = dp["params"][mod][leaf].detach().cpu().numpy().reshape(-1)
        want = ref[key]
        if key + "/idx" in ref.files:
            got = got[ref[key + "/idx"]]
        _close(got, want.reshape(-1), rtol=1e-9, what=key)
        n_checked += 1
    assert n_checked == 28  # 8 Dense x (kernel, bias) + 6 LayerNorm x (scale, bias)


def test_vs_oracle_larger_grid(G):
    wl = synthetic.make_workload(n_grid=4096, n_ao=40, n_occ=6, seed=21, box_angstrom=7.0, centre_box_angstrom=5.0)
    ao, g1, g2 = O.eval_ao_planes(wl.basis, wl.coords)
    rho = np.einsum("sab,ra,rb->rs", wl.rdm1, ao, ao)
    ehf = synthetic.make_ehf(wl.n_grid, 8, rho, n_omega=2)
    params = synthetic.glorot_params(seed=3)
    e_ref, v_ref, dp_ref = O.xc_energy_and_grads("DM21", wl.rdm1, ao, g1, g2, wl.weights, params=params, ehf=ehf,
                                                 want_param_grads=True)
    mol = _molecule(G, ao, g1, g2, wl.weights, wl.rdm1, ehf)
    e, v, dp = _dm21(G).xc_energy_and_grads_params(_params(3), mol)
    assert abs(float(e) - e_ref) <= RTOL * abs(e_ref), (float(e), e_ref)
    _close(v, v_ref, what="V_xc")
    for mod, d in dp_ref["params"].items():
        for leaf, g in d.items():
            _close(dp["params"][mod][leaf], g, rtol=1e-9, what=f"{mod}/{leaf}")


def test_finite_differences(G, ref):
    """dE/dtheta and dE/dD against central differences of the device energy."""
    mol = _molecule(G, ref["ao"], ref["grad_ao"], ref["grad2_ao"], ref["weights"], ref["rdm1"], ref["ehf"])
    f = _dm21(G)
    params = _params(5)
    e0, v, dp = f.xc_energy_and_grads_params(params, mol)
    rng = np.random.default_rng(0)
    probes = [("Dense_0", "kernel"), ("Dense_3", "kernel"), ("LayerNorm_2", "scale"), ("LayerNorm_5", "bias"),
              ("Dense_7", "kernel"), ("Dense_7", "bias"), ("Dense_1", "bias")]
    for mod, leaf in probes:
        base = params["params"][mod][leaf]
        idx = tuple(int(rng.integers(0, s)) for s in base.shape)
        h = 1e-5 * max(1.0, abs(float(base[idx])))
        vals = []
        for sgn in (1.0, -1.0):
            p = {"params": {k: dict(d) for k, d in params["params"].items()}}
            t = base.clone()
            t[idx] += sgn * h
            p["params"][mod][leaf] = t
            vals.append(float(f.xc_energy_and_grads_params(p, mol, want_dparams=False)[0]))
        fd = (vals[0] - vals[1]) / (2 * h)
        an = float(dp["params"][mod][leaf][idx])
        assert abs(fd - an) <= 1e-6 * max(abs(an), 1e-3 * abs(float(e0))), (mod, leaf, idx, fd, an)
    # dE/dD_sab for a few entries (raw, non-symmetrised V as jax.grad gives it).
    rdm1 = torch.as_tensor(ref["rdm1"], dtype=torch.float64)
    for _ in range(4):
        s, a, b = int(rng.integers(0, 2)), int(rng.integers(0, rdm1.shape[1])), int(rng.integers(0, rdm1.shape[1]))
        h = 1e-6
        vals = []
        for sgn in (1.0, -1.0):
            d = rdm1.clone()
            d[s, a, b] += sgn * h
            m = mol.replace(rdm1=_t(d))
            vals.append(float(f.xc_energy_and_grads_params(params, m, want_dparams=False)[0]))
        fd = (vals[0] - vals[1]) / (2 * h)
        an = float(v[s, a, b])
        assert abs(fd - an) <= 1e-5 * max(abs(an), 1e-3), (s, a, b, fd, an)


def test_autograd_function(G, ref):
    """energy_xc_only is a differentiable scalar in rdm1 and in the parameter tensors."""
    mol0 = _molecule(G, ref["ao"], ref["grad_ao"], ref["grad2_ao"], ref["weights"], ref["rdm1"], ref["ehf"])
    f = _dm21(G)
    params = _params(int(ref["theta_seed"]))
    leaves = {k: {kk: t.cuda().requires_grad_(True) for kk, t in d.items()} for k, d in params["params"].items()}
    rdm1 = _t(ref["rdm1"]).requires_grad_(True)
    mol = mol0.replace(rdm1=rdm1)
    e = f.energy_xc_only({"params": leaves}, mol)
    loss = (e - 0.5) ** 2
    loss.backward()
    g = 2.0 * (float(e.detach()) - 0.5)
    _close(rdm1.grad, g * ref["vxc"], what="d loss / d rdm1")
    _close(leaves["Dense_7"]["kernel"].grad, g * ref["dtheta/Dense_7/kernel"], rtol=1e-9, what="d loss / d W_out")
    _close(leaves["LayerNorm_0"]["scale"].grad, g * ref["dtheta/LayerNorm_0/scale"], rtol=1e-9, what="d loss / d g0")


def test_mixed_contractions_with_fp64_network(G):
    """TF32x3 density/V_xc contractions feeding the FP64 network: errors vs the FP64 form."""
    wl = synthetic.make_workload(n_grid=8192, n_ao=128, n_occ=16, seed=23, box_angstrom=9.0, centre_box_angstrom=6.0)
    ao, g1, g2 = O.eval_ao_planes(wl.basis, wl.coords)
    rho = np.einsum("sab,ra,rb->rs", wl.rdm1, ao, ao)
    ehf = synthetic.make_ehf(wl.n_grid, 9, rho, n_omega=2)
    f = _dm21(G)
    out = {}
    for prec in ("fp64", "tf32x3"):
        mol = _molecule(G, ao, g1, g2, wl.weights, wl.rdm1, ehf, precision=prec)
        out[prec] = f.xc_energy_and_grads_params(_params(4), mol)
    e64, v64, d64 = out["fp64"]
    e32, v32, d32 = out["tf32x3"]
    assert abs(float(e32) - float(e64)) <= 1e-6, (float(e32), float(e64))
    assert float((v32 - v64).abs().max()) <= 2e-5 * max(1.0, float(v64.abs().max()))
    k64, k32 = d64["params"]["Dense_3"]["kernel"], d32["params"]["Dense_3"]["kernel"]
    assert float((k32 - k64).abs().max()) <= 1e-4 * float(k64.abs().max())


def test_errors(G, ref):
    mol = _molecule(G, ref["ao"], ref["grad_ao"], ref["grad2_ao"], ref["weights"], ref["rdm1"], ref["ehf"])
    f = _dm21(G)
    bad = _params()
    bad["params"]["Dense_2"]["kernel"] = bad["params"]["Dense_2"]["kernel"][:, :100]
    with pytest.raises(ValueError):
        f.xc_energy_and_grads_params(bad, mol)
    with pytest.raises(ValueError):  # reference default: HF-Fock terms need chi
        G.energy_predictor(G.DM21())(_params(), mol)


@pytest.mark.parametrize("mol_prec", ["fp64", "tf32x3"])
def test_tensor_core_network_vs_fp64_network(G, mol_prec):
    """The TF32x3 network form against the FP64 one on the same molecule: E, V_xc, dE/dtheta."""
    wl = synthetic.make_workload(n_grid=16384, n_ao=64, n_occ=8, seed=61, box_angstrom=9.0, centre_box_angstrom=6.0)
    ao, g1, g2 = O.eval_ao_planes(wl.basis, wl.coords)
    rho = np.einsum("sab,ra,rb->rs", wl.rdm1, ao, ao)
    ehf = synthetic.make_ehf(wl.n_grid, 62, rho, n_omega=2)
    mol = _molecule(G, ao, g1, g2, wl.weights, wl.rdm1, ehf, precision=mol_prec)
    out = {}
    for prec in ("fp64", "tf32x3"):
        f = _dm21(G)
        f.precision = prec
        out[prec] = f.xc_energy_and_grads_params(_params(9), mol)
    assert mol.resident().status() == 0
    (e64, v64, d64), (etc, vtc, dtc) = out["fp64"], out["tf32x3"]
    de = abs(float(etc) - float(e64))
    dv = float((vtc - v64).abs().max()) / float(v64.abs().max())
    print("E", float(e64), "|dE|", de, "rel dV", dv)
    assert de <= 1e-6 * max(1.0, abs(float(e64)))
    assert dv <= 1e-5
    worst = 0.0
    for mod, d in d64["params"].items():
        for leaf, g in d.items():
            err = float((dtc["params"][mod][leaf] - g).abs().max()) / max(float(g.abs().max()), 1e-300)
            worst = max(worst, err)
            assert err <= 1e-4, (mod, leaf, err)
    print("worst rel d theta", worst)
