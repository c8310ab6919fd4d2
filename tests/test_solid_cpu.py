"""The oracle's k-point (Solid) path against the fixture of the reference's own code (no GPU).

tests/golden/make_golden_solid.py ran grad_dft/solid.py and train.py's predict
unchanged (torch stand-ins for jax, JAX's complex-gradient convention) on
Bloch-phased AOs; oracle/solid.py must reproduce densities, the Coulomb
potential, the non-XC energy and predict's (E, F).
"""
import numpy as np
import pytest
import torch

import oracle.solid as OSd


def _same(a, b, rtol=1e-13):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape
    nan = np.isnan(b)
    assert np.array_equal(np.isnan(a), nan)
    if (~nan).any():
        assert np.max(np.abs(a[~nan] - b[~nan])) <= rtol * max(np.max(np.abs(b[~nan])), 1e-300)


@pytest.mark.parametrize("case", ["solid", "solid_small_k"])
def test_densities_and_coulomb(golden, case):
    g = golden(case)
    rho, grad, lapl, tau = OSd.solid_features(torch.as_tensor(g["rdm1"]), g["ao"], g["grad_ao"], g["grad2_ao"],
                                              g["kweights"])
    _same(rho.numpy(), g["rho"])
    _same(grad.numpy(), g["grad_rho"])
    _same(lapl.numpy(), g["lapl"])
    _same(tau.numpy(), g["tau"])
    _same(OSd.solid_coulomb(g["rep"], g["rdm1"], g["kweights"]), g["vj"])
    nonxc = OSd.solid_nonxc(g["rdm1"], g["h1e"], g["rep"], float(g["nuclear_repulsion"]), g["kweights"])
    assert abs(nonxc - float(g["nonxc"])) <= 1e-13 * abs(float(g["nonxc"]))


@pytest.mark.parametrize("name", ["LSDA", "B88", "LYP", "PW92", "VWN"])
@pytest.mark.parametrize("case", ["solid", "solid_small_k"])
def test_predict(golden, name, case):
    g = golden(case)
    E, F = OSd.solid_predict(name, g["rdm1"], g["ao"], g["grad_ao"], g["grad2_ao"], g["weights"], g["kweights"],
                             g["h1e"], g["rep"], float(g["nuclear_repulsion"]))
    assert abs(E - float(g[f"E_{name}"])) <= 1e-13 * abs(float(g[f"E_{name}"]))
    _same(F, g[f"F_{name}"])


@pytest.mark.parametrize("name", ["LSDA", "B88"])
def test_scf_loop(golden, name):
    """diff_simple_scf_loop with a Solid (evaluate.py:256-344), run by the reference for the fixture."""
    g = golden("solid_scf")
    E, D, F, mo_e = OSd.solid_scf_loop(name, g["rdm1"], g["mo_occ_init"], g["ao"], g["grad_ao"], g["grad2_ao"],
                                       g["weights"], g["kweights"], g["h1e"], g["s1e"], g["rep"],
                                       float(g["nuclear_repulsion"]), int(g["cycles"]))
    assert abs(E - float(g[f"energy_{name}"])) <= 1e-12 * abs(float(g[f"energy_{name}"]))
    _same(D, g[f"rdm1_{name}"], 1e-10)
    _same(F, g[f"fock_{name}"], 1e-10)
    _same(mo_e, g[f"mo_energy_{name}"], 1e-10)
