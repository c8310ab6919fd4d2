"""Generate the golden fixtures by running the reference's own ``grad_dft`` source.

Usage (needs the reference checkout; this is not run by the tests):

    python tests/golden/make_golden.py /root/reference

The reference's dependencies (jax, flax, ...) are absent, so ``jaxshim``
supplies torch-float64 stand-ins; the reference modules ``molecule.py``,
``functional.py``, ``popular_functionals.py`` and ``train.py`` are executed
unchanged.  Inputs come from the seeded synthetic generator; everything the
reference computes from them is written to ``tests/golden/*.npz``.
"""
from __future__ import annotations

import functools
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

import jaxshim  # noqa: E402
from graddft_gb300 import synthetic  # noqa: E402
from oracle.ao_numpy import eval_ao_planes  # noqa: E402
from oracle import oracle as O  # noqa: E402  (test coefficient rows only)

F64 = torch.float64

# torch's Tensor.transpose takes two dims; the reference calls transpose(perm) (train.py:157,162)
# and transpose(*axes) (molecule.py:613).
_orig_transpose = torch.Tensor.transpose


def _transpose(self, *dims):
    if len(dims) == 1 and isinstance(dims[0], (tuple, list)):
        return self.permute(*dims[0])
    if len(dims) > 2:  # jnp's transpose(*axes) (molecule.py:613)
        return self.permute(*dims)
    return _orig_transpose(self, *dims)


CASES = {
    # name: (n_grid, n_ao, n_occ, seed, grid box (A), centre box (A))
    "compact": (512, 20, 4, 11, 6.0, 4.0),
    "tails": (384, 16, 3, 12, 20.0, 12.0),
    "dm21": (256, 16, 3, 13, 6.0, 4.0),
    "hf": (320, 18, 4, 14, 6.0, 4.0),
}


def _inputs(case):
    n_grid, n_ao, n_occ, seed, box, cbox = CASES[case]
    wl = synthetic.make_workload(n_grid, n_ao, n_occ, seed, box_angstrom=box, centre_box_angstrom=cbox)
    ao, g1, g2 = eval_ao_planes(wl.basis, wl.coords)
    rng = np.random.default_rng(seed + 1000)
    h = rng.standard_normal((n_ao, n_ao))
    h1e = 0.5 * (h + h.T)
    eri = rng.standard_normal((n_ao, n_ao, n_ao, n_ao)) * 0.01
    eri = eri + eri.transpose(1, 0, 2, 3)
    eri = eri + eri.transpose(0, 1, 3, 2)
    eri = eri + eri.transpose(2, 3, 0, 1)
    return wl, ao, g1, g2, h1e, eri


def _molecule(ref, wl, ao, g1, g2, h1e, eri):
    M = ref.molecule
    t = lambda x: torch.as_tensor(np.asarray(x), dtype=F64)  # noqa: E731
    grid = M.Grid(coords=t(wl.coords), weights=t(wl.weights))
    n = wl.n_ao
    return M.Molecule(
        grid=grid, atom_index=torch.zeros(1, dtype=torch.int64), nuclear_pos=torch.zeros(1, 3, dtype=F64),
        ao=t(ao), grad_ao=t(g1), grad_n_ao={1: t(g1), 2: t(g2)}, rdm1=t(wl.rdm1),
        nuclear_repulsion=torch.tensor(1.25, dtype=F64), h1e=t(h1e), vj=torch.zeros(2, n, n, dtype=F64),
        mo_coeff=torch.zeros(2, n, n, dtype=F64), mo_occ=torch.zeros(2, n, dtype=F64),
        mo_energy=torch.zeros(2, n, dtype=F64), rep_tensor=t(eri),
    )


def _raw_xc(ref, functional, params, molecule):
    """The body of ``xc_energy_and_grads`` (train.py:86-121) through the reference's own methods."""
    jax = sys.modules["jax"]

    def f(params, rdm1, atoms):
        atoms = atoms.replace(rdm1=rdm1)
        densities = functional.compute_densities(atoms)
        cinputs = functional.compute_coefficient_inputs(atoms)
        return functional.xc_energy(params, atoms.grid, cinputs, densities)

    e, v = jax.value_and_grad(f, argnums=1)(params, molecule.rdm1, molecule)
    return e.detach().numpy(), v.detach().numpy()


def main(root):
    torch.Tensor.transpose = _transpose
    ref = jaxshim.load_reference(root)
    pop, fun = ref.popular, ref.functional
    jnp = sys.modules["jax.numpy"]
    out_files = []

    for case in ("compact", "tails"):
        wl, ao, g1, g2, h1e, eri = _inputs(case)
        mol = _molecule(ref, wl, ao, g1, g2, h1e, eri)
        res = dict(ao=ao, grad_ao=g1, grad2_ao=g2, weights=wl.weights, rdm1=wl.rdm1, h1e=h1e, eri=eri,
                   coords=wl.coords, basis=wl.basis.packed())
        with torch.no_grad():
            res["rho"] = mol.density().numpy()
            res["grad_rho"] = mol.grad_density().numpy()
            res["lapl_rho"] = mol.lapl_density().numpy()
            res["tau"] = mol.kinetic_density().numpy()
            res["ed_lsda"] = pop.lsda_density(mol).numpy()
            res["ed_b88"] = pop.b88_density(mol).numpy()
            res["ed_vwn"] = pop.vwn_density(mol).numpy()
            res["ed_lyp"] = pop.lyp_density(mol).numpy()
            res["ed_pw92"] = pop.pw92_densities(mol).numpy()
            res["ed_b3lyp_exhf"] = pop.b3lyp_exhf_densities(mol).numpy()
            rho = mol.density()
            grad_rho = mol.grad_density()
            tau = mol.kinetic_density()
            res["dm21_cinputs"] = fun.dm21_coefficient_inputs(mol).numpy()
            res["dm21_densities_lda"] = fun.dm21_densities(mol, "LDA").numpy()
            res["dm21_densities_mgga"] = fun.dm21_densities(mol, "MGGA").numpy()
            res["densities_mgga"] = fun.densities(mol, "MGGA").numpy()
            res["dm21_densities_gga"] = fun.dm21_densities(mol, "GGA").numpy()
            res["densities_lda"] = fun.densities(mol, "LDA").numpy()
            res["densities_gga"] = fun.densities(mol, "GGA").numpy()
        # The documented dict functional_type (functional.py:548-556): the reference's code binds
        # u_range / w_range only for a string (:575-585), so it raises for a dict.
        try:
            fun.dm21_densities(mol, {"u_range": range(0, 2), "w_range": range(0, 2)})
            res["dict_type_raises"] = np.array(0)
        except UnboundLocalError:
            res["dict_type_raises"] = np.array(1)
        ehf = synthetic.make_ehf(wl.n_grid, 5, rho.numpy(), n_omega=2)
        res["ehf"] = ehf
        params = {"params": {}}
        functionals = {
            "LSDA": pop.LSDA, "B88": pop.B88, "VWN": pop.VWN, "LYP": pop.LYP, "PW92": pop.PW92,
            "BLYP": fun.Functional(coefficients=lambda self, *_: jnp.array([[1.0]]),
                                   energy_densities=lambda m, *a, **k: jnp.concatenate(
                                       (pop.b88_density(m), pop.lyp_density(m)), axis=1)),
            # B3LYP with the HF column supplied as a stop-gradient input (no chi tensor here).
            "B3LYP": fun.Functional(coefficients=pop.b3lyp_coefficients,
                                    energy_densities=pop.b3lyp_exhf_densities,
                                    nograd_densities=lambda m, *a, **k: torch.as_tensor(ehf[:1]),
                                    combine_densities=pop.b3lyp_combine),
        }
        # Constant rows on the feature powers, selected as the reference's examples select them
        # (energy_densities=partial(dm21_densities, functional_type=...)).
        for name, fn_, ftype, coeffs in (("DM21_GGA", fun.dm21_densities, "GGA", O.DM21_GGA_COEFFS),
                                         ("DM21_MGGA", fun.dm21_densities, "MGGA", O.DM21_MGGA_COEFFS),
                                         ("DENS_GGA", fun.densities, "GGA", O.DENS_GGA_COEFFS),
                                         ("DENS_MGGA", fun.densities, "MGGA", O.DENS_MGGA_COEFFS)):
            functionals[name] = fun.Functional(
                coefficients=(lambda c: (lambda self, *_: jnp.array([c])))(list(coeffs)),
                energy_densities=functools.partial(fn_, functional_type=ftype))
        for name, f in functionals.items():
            e, v = _raw_xc(ref, f, params, mol)
            res[f"exc_{name}"] = e
            res[f"vxc_{name}"] = v
            if name in ("LSDA", "B88", "BLYP"):
                E, F = ref.train.energy_predictor(f)(params, mol)
                res[f"predict_E_{name}"] = E.detach().numpy()
                res[f"predict_F_{name}"] = F.detach().numpy()
        path = os.path.join(HERE, f"ref_{case}.npz")
        np.savez_compressed(path, **res)
        out_files.append(path)

    # DM21-style neural functional with stop-gradient HF inputs (config-3 shape, small grid).
    wl, ao, g1, g2, h1e, eri = _inputs("dm21")
    mol = _molecule(ref, wl, ao, g1, g2, h1e, eri)
    with torch.no_grad():
        rho = mol.density().numpy()
    ehf = synthetic.make_ehf(wl.n_grid, 6, rho, n_omega=2)
    ehf_t = torch.as_tensor(ehf)
    dm21 = fun.DM21(densitygrads=None, coefficient_input_grads=None,
                    nograd_densities=lambda atoms, *_, **__: ehf_t,
                    nograd_coefficient_inputs=lambda atoms, *_, **__: ehf_t)
    np_params = synthetic.glorot_params(seed=7)
    params = {"params": {k: {kk: torch.as_tensor(vv) for kk, vv in v.items()} for k, v in np_params["params"].items()}}
    e, v = _raw_xc(ref, dm21, params, mol)
    jax = sys.modules["jax"]

    def exc_of_params(p):
        densities = dm21.compute_densities(mol)
        cinputs = dm21.compute_coefficient_inputs(mol)
        return dm21.xc_energy(p, mol.grid, cinputs, densities)

    dtheta = jax.grad(exc_of_params)(params)
    with torch.no_grad():
        cin = dm21.compute_coefficient_inputs(mol)
        coeffs = dm21.apply(params, cin)
        dens = dm21.compute_densities(mol)
    sel = np.random.default_rng(99)
    res = dict(ao=ao, grad_ao=g1, grad2_ao=g2, weights=wl.weights, rdm1=wl.rdm1, ehf=ehf,
               exc=e, vxc=v, cinputs=cin.numpy(), coefficients=coeffs.numpy(), densities=dens.numpy(),
               theta_seed=np.array(7))
    for k, d in dtheta["params"].items():
        for kk, g in d.items():
            g = g.detach().numpy()
            if g.size > 4096:
                idx = np.sort(sel.choice(g.size, 2048, replace=False))
                res[f"dtheta/{k}/{kk}/idx"] = idx
                res[f"dtheta/{k}/{kk}"] = g.reshape(-1)[idx]
            else:
                res[f"dtheta/{k}/{kk}"] = g
    path = os.path.join(HERE, "ref_dm21.npz")
    np.savez_compressed(path, **res)
    out_files.append(path)
    # B3LYP with its exact-exchange terms from a chi tensor (molecule.py:153-300,
    # popular_functionals.py:345-391, train.py:165-213): predict() runs the
    # reference's HF_energy_density and HF_density_grad_2_Fock unchanged.
    wl, ao, g1, g2, h1e, eri = _inputs("hf")
    mol = _molecule(ref, wl, ao, g1, g2, h1e, eri)
    omegas = np.array([0.0, 0.4])
    chi = synthetic.make_chi(ao, wl.rdm1, n_omega=2, seed=15)
    mol = mol.replace(chi=torch.as_tensor(chi), omegas=torch.as_tensor(omegas))
    res = dict(ao=ao, grad_ao=g1, grad2_ao=g2, weights=wl.weights, rdm1=wl.rdm1, h1e=h1e, eri=eri, chi=chi,
               omegas=omegas)
    with torch.no_grad():
        res["ehf"] = mol.HF_energy_density(list(omegas)).numpy()
        res["ehf_w0"] = mol.HF_energy_density([0.0]).numpy()
    params = {"params": {}}
    E, F = ref.train.energy_predictor(pop.B3LYP)(params, mol)
    res["predict_E_B3LYP"] = E.detach().numpy()
    res["predict_F_B3LYP"] = F.detach().numpy()
    ehf0 = mol.HF_energy_density([0.0]).detach()
    vexpl = pop.b3lyp_hfgrads(pop.B3LYP, params, mol, ehf0, None, pop.b3lyp_exhf_densities(mol))
    res["b3lyp_hfgrads"] = vexpl.detach().numpy()
    # DM21 with its default slots: HF inputs and densities from chi, and both
    # HF Fock terms (functional.py:677-785) in predict.
    dm21 = fun.DM21()
    np_params = synthetic.glorot_params(seed=7)
    params = {"params": {k: {kk: torch.as_tensor(vv) for kk, vv in v.items()} for k, v in np_params["params"].items()}}
    E, F = ref.train.energy_predictor(dm21)(params, mol)
    res["predict_E_DM21"] = E.detach().numpy()
    res["predict_F_DM21"] = F.detach().numpy()
    with torch.no_grad():
        ehf = mol.HF_energy_density(jnp.array([0.0, 0.4]))
        dens_wout = dm21.energy_densities(mol)
        cin_wout = dm21.coefficient_inputs(mol)
    cin = dm21.combine_inputs(cin_wout, ehf)
    dens = dm21.combine_densities(dens_wout, ehf)
    res["dm21_hfgrads_densities"] = fun.dm21_hfgrads_densities(dm21, params, mol, ehf, cin, dens_wout).detach().numpy()
    res["dm21_hfgrads_cinputs"] = fun.dm21_hfgrads_cinputs(dm21, params, mol, ehf, cin_wout, dens).detach().numpy()
    res["theta_seed"] = np.array(7)
    path = os.path.join(HERE, "ref_hf.npz")
    np.savez_compressed(path, **res)
    out_files.append(path)
    # Config 1's stand-in (its PySCF H2O / def2-TZVP inputs are not available): unrestricted B3LYP evaluated
    # non-self-consistently on a fixed D at n_ao = 43 (popular_functionals.py:384-391), its HF column from a
    # chi tensor: E_xc and V_xc of xc_energy_and_grads (train.py:86-121) and the explicit HF Fock term
    # (popular_functionals.py:352-372).  The inputs are regenerated from seeds (oracle/cases.py), so only
    # the reference's outputs are stored.
    from oracle.cases import b3lyp43_inputs

    wl, ao, g1, g2, chi, omegas = b3lyp43_inputs()
    n = wl.n_ao
    mol = _molecule(ref, wl, ao, g1, g2, np.zeros((n, n)), np.zeros((1, 1, 1, 1)))
    mol = mol.replace(chi=torch.as_tensor(chi), omegas=torch.as_tensor(omegas))
    params = {"params": {}}
    e, v = _raw_xc(ref, pop.B3LYP, params, mol)
    with torch.no_grad():
        ehf0 = mol.HF_energy_density([0.0])
    vexpl = pop.b3lyp_hfgrads(pop.B3LYP, params, mol, ehf0.detach(), None, pop.b3lyp_exhf_densities(mol))
    res = dict(exc=e, vxc=v, ehf=ehf0.numpy(), b3lyp_hfgrads=vexpl.detach().numpy(), n_ao=np.array(n),
               n_grid=np.array(wl.n_grid))
    path = os.path.join(HERE, "ref_b3lyp43.npz")
    np.savez_compressed(path, **res)
    out_files.append(path)
    # diff_scf_loop (evaluate.py:917-1038) with JittableDiis (:1041-1210): the
    # final energy, density matrix and dE/dtheta through all iterations, DM21
    # with stop-gradient HF inputs, 12 cycles (past the 10-entry DIIS history).
    ev = jaxshim.load_scf(root, ref)
    wl, ao, g1, g2, _, _ = _inputs("dm21")
    n = wl.n_ao
    sysm = synthetic.make_scf_system(n, 3, naux=32, seed=17)
    eri = np.einsum("Ppq,Prs->pqrs", sysm.df_tensor, sysm.df_tensor)
    mol = _molecule(ref, wl, ao, g1, g2, sysm.h1e, eri)
    tt = lambda x: torch.as_tensor(np.asarray(x), dtype=F64)  # noqa: E731
    mol = mol.replace(rdm1=tt(sysm.rdm1), s1e=tt(sysm.s1e), mo_occ=tt(sysm.mo_occ),
                      nuclear_repulsion=tt(sysm.nuclear_repulsion))
    rho = np.einsum("sab,ra,rb->rs", sysm.rdm1, ao, ao)
    ehf_t = torch.as_tensor(synthetic.make_ehf(wl.n_grid, 18, rho, n_omega=2))
    dm21 = fun.DM21(densitygrads=None, coefficient_input_grads=None,
                    nograd_densities=lambda atoms, *_, **__: ehf_t,
                    nograd_coefficient_inputs=lambda atoms, *_, **__: ehf_t)
    np_params = synthetic.glorot_params(seed=19)
    params = {"params": {k: {kk: torch.as_tensor(vv) for kk, vv in v.items()} for k, v in np_params["params"].items()}}
    cycles = 12
    loop = ev.diff_scf_loop(dm21, cycles=cycles)
    jax = sys.modules["jax"]
    out = {}

    def final_energy(p):
        m = loop(p, mol)
        out["mol"] = m
        return m.energy

    dtheta = jax.grad(final_energy)(params)
    m = out["mol"]
    res = dict(ao=ao, grad_ao=g1, grad2_ao=g2, weights=wl.weights, ehf=ehf_t.numpy(), h1e=sysm.h1e, s1e=sysm.s1e,
               df_tensor=sysm.df_tensor, rdm1_init=sysm.rdm1, mo_occ=sysm.mo_occ,
               nuclear_repulsion=np.array(sysm.nuclear_repulsion), theta_seed=np.array(19), cycles=np.array(cycles),
               energy=m.energy.detach().numpy(), rdm1=m.rdm1.detach().numpy(), fock=m.fock.detach().numpy())
    sel = np.random.default_rng(98)
    for k, d in dtheta["params"].items():
        for kk, g in d.items():
            g = g.detach().numpy()
            if g.size > 4096:
                idx = np.sort(sel.choice(g.size, 2048, replace=False))
                res[f"dtheta/{k}/{kk}/idx"] = idx
                res[f"dtheta/{k}/{kk}"] = g.reshape(-1)[idx]
            else:
                res[f"dtheta/{k}/{kk}"] = g
    path = os.path.join(HERE, "ref_scf_diis.npz")
    np.savez_compressed(path, **res)
    out_files.append(path)
    torch.Tensor.transpose = _orig_transpose
    for p in out_files:
        print(p, os.path.getsize(p))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
