"""The oracle's nu integrals and chi (no GPU).

nu_ab(C) = int phi_a phi_b erf(omega |r - C|)/|r - C| is PySCF's int1e_grids in
the reference (external/_hf_density.py:17-120); chi is generate_chi_tensor
(interface/pyscf.py:1067-1126).  PySCF is absent, so the oracle's
McMurchie-Davidson integrals are pinned by direct quadrature around C, by the
closed form of s-type pairs and by the Boys function at high precision; the chi
assembly is pinned by the fixture made from the reference's own functions
(tests/golden/make_golden_chi.py).
"""
import math

import numpy as np
import pytest
from scipy.special import erf

from oracle import nu as ONU
from oracle import shells as OS


def _fixture_shells(g):
    return [(g[f"shell{i}/centre"], int(g[f"shell{i}/l"]), g[f"shell{i}/exps"], g[f"shell{i}/coefs"], None)
            for i in range(int(g["n_shell"]))]


def test_boys_against_high_precision():
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.dps = 40
    T = np.array([0.0, 1e-8, 0.3, 0.99, 1.0, 2.5, 7.0, 19.9, 35.0, 59.7, 75.0])
    F = ONU.boys(8, T)
    for n in range(9):
        for k, t in enumerate(T):
            ref = mpmath.quad(lambda u: u ** (2 * n) * mpmath.exp(-t * u * u), [0, 1])
            assert abs(F[n, k] - float(ref)) <= 2e-15 * float(ref), (n, t)


def test_ss_closed_form():
    """Two normalised s primitives: nu = N_a N_b K (pi/p)^(3/2) erf(sqrt(mu) R)/R."""
    a, b = 1.3, 0.45
    A, B = np.array([0.2, -0.1, 0.4]), np.array([-0.6, 0.5, 0.1])
    C = np.array([[0.3, 0.3, -0.2], [2.0, -1.0, 0.5], [0.2, -0.1, 0.4]])
    ca = OS.normalise_contraction(0, [a], [[1.0]])
    cb = OS.normalise_contraction(0, [b], [[1.0]])
    shells = [(A, 0, [a], ca, None), (B, 0, [b], cb, None)]
    y00 = 1 / math.sqrt(4 * math.pi)
    p = a + b
    P = (a * A + b * B) / p
    K = math.exp(-a * b / p * np.sum((A - B) ** 2))
    for omega in (0.0, 0.4, 2.0):
        mu = p if omega == 0 else p * omega ** 2 / (p + omega ** 2)
        R = np.linalg.norm(P[None, :] - C, axis=1)
        ref = ca[0, 0] * cb[0, 0] * y00 * y00 * K * (math.pi / p) ** 1.5 * erf(math.sqrt(mu) * R) / R
        got = ONU.nu_integrals(shells, C, omega)[:, 0, 1]
        assert np.max(np.abs(got - ref) / np.abs(ref)) < 1e-13


def _quadrature_nu(shells, C, omega, n_r=140, n_t=48, n_p=96, s_max=11.0):
    x, wx = np.polynomial.legendre.leggauss(n_r)
    s = s_max * (x + 1) / 2
    ws = wx * s_max / 2
    ct, wt = np.polynomial.legendre.leggauss(n_t)
    ph = 2 * np.pi * np.arange(n_p) / n_p
    st = np.sqrt(1 - ct * ct)
    dirs = np.stack([st[:, None] * np.cos(ph)[None, :], st[:, None] * np.sin(ph)[None, :],
                     np.repeat(ct[:, None], n_p, axis=1)], axis=-1).reshape(-1, 3)
    wd = (wt[:, None] * np.full(n_p, 2 * np.pi / n_p)[None, :]).reshape(-1)
    kern = s * (erf(omega * s) if omega > 0 else 1.0) * ws  # s^2 * v(s) ds, v(s) = erf(omega s)/s
    out = None
    for k in range(n_r):
        pts = C[None, :] + s[k] * dirs
        ao, _, _ = OS.eval_shells(shells, pts)
        blk = np.einsum("p,pa,pb->ab", wd * kern[k], ao, ao)
        out = blk if out is None else out + blk
    return out


@pytest.mark.parametrize("omega", [0.0, 0.4])
def test_integrals_against_quadrature(omega):
    g = np.random.default_rng(5)
    shells = []
    for l in (0, 1, 2, 3):
        e = [1.1, 0.55] if l == 0 else [0.8]
        c = OS.normalise_contraction(l, e, np.ones((len(e), 1)))
        shells.append((g.uniform(-0.6, 0.6, 3), l, np.asarray(e), c, None))
    C = np.array([[0.15, -0.2, 0.1], [0.9, 0.4, -0.5]])
    nu = ONU.nu_integrals(shells, C, omega)
    for k in range(C.shape[0]):
        q = _quadrature_nu(shells, C[k], omega)
        assert np.max(np.abs(nu[k] - q)) < 2e-9 * np.max(np.abs(q)), k
    assert np.allclose(nu, nu.transpose(0, 2, 1), rtol=0, atol=0)


def test_large_omega_tends_to_coulomb():
    g = np.random.default_rng(6)
    shells = [(g.uniform(-1, 1, 3), l, [0.9], OS.normalise_contraction(l, [0.9], [[1.0]]), None) for l in (0, 1, 2)]
    C = g.uniform(-2, 2, (5, 3))
    full = ONU.nu_integrals(shells, C, 0.0)
    att = ONU.nu_integrals(shells, C, 1e4)
    assert np.max(np.abs(full - att)) < 1e-7 * np.max(np.abs(full))


def test_oracle_chi_matches_reference_fixture(golden):
    """The reference's generate_chi_tensor (run by make_golden_chi.py) on the oracle's integrals."""
    g = golden("chi")
    shells = _fixture_shells(g)
    nus = [ONU.nu_integrals(shells, g["coords"], w) for w in g["omegas"]]
    chi = ONU.generate_chi(g["rdm1"], g["ao"], nus)
    assert chi.shape == g["chi"].shape == (150, 2, 2, 30)
    assert np.max(np.abs(chi - g["chi"])) <= 1e-13 * np.max(np.abs(g["chi"]))
    assert np.max(np.abs(nus[1][:16] - g["nu04_first16"])) == 0.0
