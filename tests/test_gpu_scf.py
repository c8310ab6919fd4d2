"""GPU parity of the second-order adjoint (Hessian-vector product of E_xc) and
of the differentiable SCF loop, against the oracle's torch double-backward."""
import numpy as np
import pytest
import torch

import oracle as O
from graddft_gb300 import synthetic

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    b = np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module")
def G(built_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import graddft_gb300 as G

    return G


def _t(x):
    return torch.as_tensor(np.asarray(x), dtype=torch.float64, device="cuda")


def _params(seed):
    p = synthetic.glorot_params(seed=seed)
    return {"params": {k: {kk: torch.as_tensor(v) for kk, v in d.items()} for k, d in p["params"].items()}}


def _dm21(G):
    hf = lambda atoms, *_, **__: atoms.ehf  # noqa: E731
    return G.DM21(densitygrads=None, coefficient_input_grads=None, nograd_densities=hf, nograd_coefficient_inputs=hf)


def _case(n_grid=2048, n_ao=24, n_occ=4, seed=31):
    wl = synthetic.make_workload(n_grid, n_ao, n_occ, seed=seed, box_angstrom=7.0, centre_box_angstrom=5.0)
    ao, g1, g2 = O.eval_ao_planes(wl.basis, wl.coords)
    rho = np.einsum("sab,ra,rb->rs", wl.rdm1, ao, ao)
    ehf = synthetic.make_ehf(n_grid, seed + 1, rho, n_omega=2)
    return wl, ao, g1, g2, ehf


def _molecule(G, ao, g1, g2, w, rdm1, ehf, precision="fp64", **extra):
    return G.Molecule(grid=G.Grid(coords=None, weights=_t(w)), atom_index=None, nuclear_pos=None, ao=_t(ao),
                      grad_ao=_t(g1), grad_n_ao={2: _t(g2)}, rdm1=_t(rdm1), nuclear_repulsion=0.0, h1e=None,
                      vj=None, mo_coeff=None, mo_occ=None, mo_energy=None, ehf=_t(ehf), precision=precision,
                      **extra)


def test_hvp_vs_oracle(G):
    wl, ao, g1, g2, ehf = _case()
    params = synthetic.glorot_params(seed=6)
    tangent = np.random.default_rng(5).standard_normal(wl.rdm1.shape)
    L_ref, hD_ref, hp_ref = O.xc_hvp("DM21", wl.rdm1, ao, g1, g2, wl.weights, tangent, params=params, ehf=ehf)
    mol = _molecule(G, ao, g1, g2, wl.weights, wl.rdm1, ehf)
    f = _dm21(G)
    net = f.network()
    r = mol.resident()
    flat = net.flatten(_params(6), r.device)
    L, hD, hp = r.neural_xc_hvp(mol._rdm1(), net, flat, mol.ehf, _t(tangent), want_value=True)
    assert r.status() == 0
    # <G, V> from the first-order path
    _, v, _ = r.neural_xc_energy_and_grads(mol._rdm1(), net, flat, mol.ehf)
    assert abs(float(L) - L_ref) <= 1e-10 * abs(L_ref), (float(L), L_ref)
    assert abs(float((v * _t(tangent)).sum()) - L_ref) <= 1e-10 * abs(L_ref)
    assert _rel(hD, hD_ref) <= 1e-9, _rel(hD, hD_ref)
    hp_tree = net.unflatten(hp)
    for mod, d in hp_ref["params"].items():
        for leaf, g in d.items():
            err = _rel(hp_tree["params"][mod][leaf], g)
            assert err <= 1e-8, (mod, leaf, err)


def test_hvp_vs_finite_differences_of_vxc(G):
    """<dL/dD, H> against central differences of <G, V_xc(D + h H)> on the device."""
    wl, ao, g1, g2, ehf = _case(seed=41)
    mol = _molecule(G, ao, g1, g2, wl.weights, wl.rdm1, ehf)
    f = _dm21(G)
    net = f.network()
    r = mol.resident()
    flat = net.flatten(_params(8), r.device)
    rng = np.random.default_rng(9)
    tangent, H = _t(rng.standard_normal(wl.rdm1.shape)), rng.standard_normal(wl.rdm1.shape)
    _, hD, _ = r.neural_xc_hvp(mol._rdm1(), net, flat, mol.ehf, tangent, want_dparams=False)
    h = 1e-5
    vals = []
    for sgn in (1.0, -1.0):
        _, v, _ = r.neural_xc_energy_and_grads(_t(wl.rdm1 + sgn * h * H), net, flat, mol.ehf)
        vals.append(float((v * tangent).sum()))
    fd = (vals[0] - vals[1]) / (2 * h)
    an = float((hD * _t(H)).sum())
    # Central differences of a function with abs_clip / clip kinks agree to ~1e-5
    # (the oracle's double-backward above is the exact check).
    assert abs(fd - an) <= 1e-4 * abs(an), (fd, an)


def test_pair_autograd_second_order(G):
    """(E, V) from xc_energy_and_potential carry second-order gradients through V."""
    wl, ao, g1, g2, ehf = _case(seed=51)
    params = synthetic.glorot_params(seed=4)
    tangent = np.random.default_rng(3).standard_normal(wl.rdm1.shape)
    L_ref, hD_ref, hp_ref = O.xc_hvp("DM21", wl.rdm1, ao, g1, g2, wl.weights, tangent, params=params, ehf=ehf)
    e_ref, v_ref, dp_ref = O.xc_energy_and_grads("DM21", wl.rdm1, ao, g1, g2, wl.weights, params=params, ehf=ehf,
                                                 want_param_grads=True)
    rdm1 = _t(wl.rdm1).requires_grad_(True)
    mol = _molecule(G, ao, g1, g2, wl.weights, wl.rdm1, ehf).replace(rdm1=rdm1)
    tp = _params(4)
    leaves = {k: {kk: t.cuda().requires_grad_(True) for kk, t in d.items()} for k, d in tp["params"].items()}
    e, v = _dm21(G).xc_energy_and_potential({"params": leaves}, mol)
    loss = 0.5 * e + (v * _t(tangent)).sum()
    loss.backward()
    assert _rel(rdm1.grad, 0.5 * v_ref + hD_ref) <= 1e-9
    for mod, d in hp_ref["params"].items():
        for leaf, g in d.items():
            want = 0.5 * dp_ref["params"][mod][leaf] + g
            assert _rel(leaves[mod][leaf].grad, want) <= 1e-8, (mod, leaf)


def test_scf_loop_vs_oracle(G):
    n_ao, n_occ, cycles, mix = 24, 4, 3, 0.3
    wl, ao, g1, g2, _ = _case(n_grid=1024, n_ao=n_ao, n_occ=n_occ, seed=3)
    sysm = synthetic.make_scf_system(n_ao, n_occ, naux=64, seed=1)
    rho = np.einsum("sab,ra,rb->rs", sysm.rdm1, ao, ao)
    ehf = synthetic.make_ehf(wl.n_grid, 5, rho, 2)
    params = synthetic.glorot_params(seed=2)
    from oracle import scf as OS

    e_ref, g_ref, d_ref = OS.scf_energy_and_grads(params, ao, g1, g2, wl.weights, ehf, sysm.h1e, sysm.s1e,
                                                  sysm.df_tensor, sysm.nuclear_repulsion, sysm.rdm1, sysm.mo_occ,
                                                  cycles, mix)
    mol = _molecule(G, ao, g1, g2, wl.weights, sysm.rdm1, ehf, df_tensor=_t(sysm.df_tensor)).replace(
        h1e=_t(sysm.h1e), s1e=_t(sysm.s1e), nuclear_repulsion=_t(sysm.nuclear_repulsion), mo_occ=_t(sysm.mo_occ))
    tp = _params(2)
    leaves = {k: {kk: t.cuda().requires_grad_(True) for kk, t in d.items()} for k, d in tp["params"].items()}
    out = G.diff_simple_scf_loop(_dm21(G), cycles=cycles, mixing_factor=mix)({"params": leaves}, mol)
    out.energy.backward()
    assert abs(float(out.energy.detach()) - e_ref) <= 1e-10 * abs(e_ref), (float(out.energy), e_ref)
    assert _rel(out.rdm1.detach(), d_ref) <= 1e-9
    for mod, d in g_ref["params"].items():
        for leaf, g in d.items():
            err = _rel(leaves[mod][leaf].grad, g)
            assert err <= 1e-7, (mod, leaf, err)


@pytest.mark.parametrize("mol_prec", ["fp64", "tf32x3"])
def test_hvp_tensor_core_vs_fp64(G, mol_prec):
    """The mixed (tensor-core) second-order pass against the FP64 one."""
    wl, ao, g1, g2, ehf = _case(n_grid=8192, n_ao=48, n_occ=6, seed=71)
    mol = _molecule(G, ao, g1, g2, wl.weights, wl.rdm1, ehf, precision=mol_prec)
    r = mol.resident()
    tangent = _t(np.random.default_rng(7).standard_normal(wl.rdm1.shape))
    out = {}
    for prec in ("fp64", "tf32x3"):
        f = _dm21(G)
        f.precision = prec
        net = f.network()
        flat = net.flatten(_params(12), r.device)
        L, hD, hp = r.neural_xc_hvp(mol._rdm1(), net, flat, mol.ehf, tangent, want_value=True)
        out[prec] = (float(L), hD, net.unflatten(hp))
    assert r.status() == 0
    (L64, hD64, hp64), (Ltc, hDtc, hptc) = out["fp64"], out["tf32x3"]
    print("L", L64, "rel dL", abs(Ltc - L64) / abs(L64), "rel dD", _rel(hDtc, hD64.cpu().numpy()))
    assert abs(Ltc - L64) <= 1e-5 * abs(L64)
    assert _rel(hDtc, hD64.cpu().numpy()) <= 1e-4
    worst = 0.0
    for mod, d in hp64["params"].items():
        for leaf, g in d.items():
            worst = max(worst, _rel(hptc["params"][mod][leaf], g.cpu().numpy()))
    print("worst rel dtheta", worst)
    assert worst <= 1e-3


def test_scf_loop_mixed_vs_oracle(G):
    """The SCF loop with TF32x3 contractions and the tensor-core network (forward and second order)."""
    n_ao, n_occ, cycles, mix = 24, 4, 3, 0.3
    wl, ao, g1, g2, _ = _case(n_grid=1024, n_ao=n_ao, n_occ=n_occ, seed=3)
    sysm = synthetic.make_scf_system(n_ao, n_occ, naux=64, seed=1)
    rho = np.einsum("sab,ra,rb->rs", sysm.rdm1, ao, ao)
    ehf = synthetic.make_ehf(wl.n_grid, 5, rho, 2)
    params = synthetic.glorot_params(seed=2)
    from oracle import scf as OS

    e_ref, g_ref, _ = OS.scf_energy_and_grads(params, ao, g1, g2, wl.weights, ehf, sysm.h1e, sysm.s1e,
                                              sysm.df_tensor, sysm.nuclear_repulsion, sysm.rdm1, sysm.mo_occ,
                                              cycles, mix)
    mol = _molecule(G, ao, g1, g2, wl.weights, sysm.rdm1, ehf, precision="tf32x3",
                    df_tensor=_t(sysm.df_tensor)).replace(
        h1e=_t(sysm.h1e), s1e=_t(sysm.s1e), nuclear_repulsion=_t(sysm.nuclear_repulsion), mo_occ=_t(sysm.mo_occ))
    tp = _params(2)
    leaves = {k: {kk: t.cuda().requires_grad_(True) for kk, t in d.items()} for k, d in tp["params"].items()}
    f = _dm21(G)
    f.precision = "tf32x3"
    out = G.diff_simple_scf_loop(f, cycles=cycles, mixing_factor=mix)({"params": leaves}, mol)
    out.energy.backward()
    de = abs(float(out.energy.detach()) - e_ref)
    worst = max(_rel(leaves[m][l].grad, g) for m, d in g_ref["params"].items() for l, g in d.items())
    print("|dE|", de, "worst rel dtheta", worst)
    assert de <= 1e-6 * abs(e_ref)
    assert worst <= 1e-3


@pytest.mark.parametrize("precision", ["fp64", "tf32x3"])
def test_diis_scf_loop_vs_reference(G, golden, precision):
    """diff_scf_loop with JittableDiis (evaluate.py:917-1210) against the reference's own loop run on the
    same inputs (tests/golden/make_golden.py): final energy, density matrix and dE/dtheta through all
    12 iterations, past the 10-entry DIIS history."""
    g = golden("scf_diis")
    mol = _molecule(G, g["ao"], g["grad_ao"], g["grad2_ao"], g["weights"], g["rdm1_init"], g["ehf"],
                    precision=precision, df_tensor=_t(g["df_tensor"])).replace(
        h1e=_t(g["h1e"]), s1e=_t(g["s1e"]), nuclear_repulsion=_t(g["nuclear_repulsion"]), mo_occ=_t(g["mo_occ"]))
    tp = _params(int(g["theta_seed"]))
    leaves = {k: {kk: t.cuda().requires_grad_(True) for kk, t in d.items()} for k, d in tp["params"].items()}
    dm21 = _dm21(G)
    if precision == "tf32x3":
        dm21 = G.DM21(densitygrads=None, coefficient_input_grads=None, nograd_densities=dm21.nograd_densities,
                      nograd_coefficient_inputs=dm21.nograd_coefficient_inputs, precision="tf32x3")
    out = G.diff_scf_loop(dm21, cycles=int(g["cycles"]))({"params": leaves}, mol)
    out.energy.backward()
    # CDIIS solves a bordered system that grows ill-conditioned as the error
    # vectors shrink, so summation-order differences of the FP64 XC terms grow
    # over the iterations (the final energy, variational, stays at 1e-10).
    e_tol, d_tol, g_tol = (1e-10, 5e-8, 1e-8) if precision == "fp64" else (1e-7, 1e-5, 5e-6)
    e_ref = float(g["energy"])
    d_err = _rel(out.rdm1.detach(), g["rdm1"])
    print(precision, "dE", abs(float(out.energy.detach()) - e_ref) / abs(e_ref), "dD", d_err)
    assert abs(float(out.energy.detach()) - e_ref) <= e_tol * abs(e_ref), (float(out.energy), e_ref)
    assert d_err <= d_tol
    worst = 0.0
    for key in g.files:
        if not key.startswith("dtheta/") or key.endswith("/idx"):
            continue
        _, mod, leaf = key.split("/")
        got = leaves[mod][leaf].grad.detach().cpu().numpy().reshape(-1)
        if key + "/idx" in g.files:
            got = got[g[key + "/idx"]]
        err = _rel(got, g[key].reshape(-1))
        worst = max(worst, err)
        assert err <= g_tol, (key, err)
    print(precision, "max rel d(dE/dtheta) per leaf", worst)


def _simple_scf_molecule(G, g, precision):
    t = lambda x: torch.as_tensor(np.asarray(x), dtype=torch.float64, device="cuda")  # noqa: E731
    return G.Molecule(grid=G.Grid(coords=t(g["coords"]), weights=t(g["weights"])),
                      atom_index=torch.as_tensor(g["atom_index"]), nuclear_pos=None, ao=t(g["ao"]),
                      grad_ao=t(g["grad_ao"]), grad_n_ao={2: t(g["grad2_ao"])}, rdm1=t(g["rdm1"]),
                      nuclear_repulsion=float(g["nuclear_repulsion"]), h1e=t(g["h1e"]), vj=None,
                      mo_coeff=t(g["mo_coeff"]), mo_occ=t(g["mo_occ"]), mo_energy=t(g["mo_energy"]),
                      s1e=t(g["s1e"]), rep_tensor=t(g["eri"]), fock=t(np.zeros_like(g["h1e"])), charge=0,
                      precision=precision)


@pytest.mark.parametrize("name", ["B88", "LSDA"])
@pytest.mark.parametrize("precision,rtol_e,rtol_m", [("fp64", 1e-11, 1e-9), ("tf32x3", 1e-6, 2e-5)])
def test_simple_scf_loop_and_non_scf_predictor_vs_reference(G, golden, name, precision, rtol_e, rtol_m):
    """simple_scf_loop (evaluate.py:131-254) and non_scf_predictor (evaluate.py:88-126) against the
    reference's own functions (tests/golden/make_golden_simple_scf.py)."""
    g = golden("simple_scf")
    mol = _simple_scf_molecule(G, g, precision)
    fn = getattr(G, name)
    final = G.simple_scf_loop(fn, mixing_factor=float(g["mixing_factor"]), cycles=int(g["cycles"]))(
        {"params": {}}, mol)
    ref_e = float(g[f"energy_{name}"])
    assert abs(float(final.energy) - ref_e) <= rtol_e * abs(ref_e)
    for key, got in (("rdm1", final.rdm1), ("fock", final.fock), ("mo_energy", final.mo_energy)):
        ref = g[f"{key}_{name}"]
        err = float(np.max(np.abs(got.detach().cpu().numpy() - ref)))
        assert err <= rtol_m * float(np.max(np.abs(ref))), (key, err)
    nsp = G.non_scf_predictor(fn)({"params": {}}, mol)
    assert abs(float(nsp.energy) - float(g[f"nonscf_energy_{name}"])) <= rtol_e * abs(float(g[f"nonscf_energy_{name}"]))
    err = float(np.max(np.abs(nsp.fock.detach().cpu().numpy() - g[f"nonscf_fock_{name}"])))
    assert err <= rtol_m * float(np.max(np.abs(g[f"nonscf_fock_{name}"])))


def test_simple_scf_loop_charge_check(G, golden):
    """The loop's charge assertion (evaluate.py:212-220) fires when the electron count does not match."""
    g = golden("simple_scf")
    mol = _simple_scf_molecule(G, g, "fp64").replace(charge=1)
    with pytest.raises(AssertionError):
        G.simple_scf_loop(G.LSDA, cycles=2)({"params": {}}, mol)


@pytest.mark.parametrize("precision,rtol", [("fp64", 1e-9), ("tf32x3", 1e-5)])
def test_orbital_optimizers_vs_reference(G, golden, precision, rtol):
    """mol_orb_optimizer (PCA / Cholesky / ZCA whitening) and jitted_mol_orb_optimizer
    (evaluate.py:595-915) with adam(1e-2), 3 steps, against the reference's own functions."""
    g = golden("simple_scf")
    t = lambda x: torch.as_tensor(np.asarray(x), dtype=torch.float64, device="cuda")  # noqa: E731
    mol = _simple_scf_molecule(G, g, precision)
    mol = mol.replace(ao=t(g["orb/ao"]), grad_ao=t(g["orb/grad_ao"]), grad_n_ao={2: t(g["orb/grad2_ao"])},
                      s1e=t(g["orb/s1e"]), h1e=t(g["orb/h1e"]), rep_tensor=t(g["orb/eri"]),
                      mo_coeff=t(g["orb/mo_coeff"]), rdm1=t(g["orb/rdm1"]))
    for whitening in ("PCA", "Cholesky", "ZCA"):
        m = G.mol_orb_optimizer(G.B88, G.optim.adam(1e-2), cycles=3, whitening=whitening)({"params": {}}, mol)
        ref = float(g[f"orb_energy_{whitening}"])
        assert abs(float(m.energy) - ref) <= rtol * abs(ref), (whitening, float(m.energy), ref)
    m = G.jitted_mol_orb_optimizer(G.B88, G.optim.adam(1e-2), cycles=3)({"params": {}}, mol)
    ref = float(g["orb_energy_jitted"])
    assert abs(float(m.energy) - ref) <= rtol * abs(ref)


@pytest.mark.parametrize("precision,rtol_e,rtol_m", [("fp64", 1e-10, 1e-7), ("tf32x3", 1e-6, 2e-5)])
def test_scf_loop_vs_reference(G, golden, precision, rtol_e, rtol_m):
    """scf_loop (evaluate.py:355-592) with CDIIS: all cycles, with damping and level shift, and to
    convergence (with the final extra diagonalisation), against the reference's own loop."""
    g = golden("simple_scf")
    mol = _simple_scf_molecule(G, g, precision)
    runs = {"plain": dict(cycles=6, e_conv=1e-14, g_conv=1e-14),
            "shifted": dict(cycles=6, e_conv=1e-14, g_conv=1e-14, level_shift_factor=(0.1, 0.1),
                            damp_factor=(0.3, 0.3), diis_start_cycle=3),
            "converged": dict(cycles=60)}
    for key, kw in runs.items():
        final = G.scf_loop(G.B88, **kw)({"params": {}}, mol)
        ref_e = float(g[f"scf_{key}_energy"])
        assert abs(float(final.energy) - ref_e) <= rtol_e * abs(ref_e), (key, float(final.energy), ref_e)
        for part in ("rdm1", "fock"):
            ref = g[f"scf_{key}_{part}"]
            err = float(np.max(np.abs(getattr(final, part).detach().cpu().numpy() - ref)))
            assert err <= rtol_m * float(np.max(np.abs(ref))), (key, part, err)
    with pytest.raises(NotImplementedError):
        G.scf_loop(G.B88, diis_method="EDIIS")({"params": {}}, mol)
