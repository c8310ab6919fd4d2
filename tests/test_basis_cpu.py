"""Contracted Gaussian basis: host logic and the oracle's definitions (no GPU).

The reference evaluates AOs with PySCF's numint.eval_ao
(interface/pyscf.py:824, 849-852) and ao_grads (interface/pyscf.py:677-705).
PySCF is absent here; the definitions are pinned by properties: the angular
rows (exact polynomial arithmetic in graddft_gb300.basis) against an
independent fit to SciPy's spherical harmonics, orthonormality on the sphere,
unit norm of whole AOs, finite differences of the oracle's derivatives, and the
seeded synthetic basis reproduced through the general shell description.
"""
import math

import numpy as np
import pytest

import oracle as O
from oracle import shells as OS
from graddft_gb300 import basis as B
from graddft_gb300 import synthetic


@pytest.mark.parametrize("l", range(B.MAX_L + 1))
def test_solid_harmonic_rows_match_scipy(l):
    a = B.solid_harmonic_rows(l)
    b = OS.spherical_rows(l)
    assert a.shape == (2 * l + 1, B.ncart(l))
    assert np.max(np.abs(a - b)) < 1e-12 * max(1.0, np.max(np.abs(a)))


def _sphere_quadrature(n=24):
    x, w = np.polynomial.legendre.leggauss(n)  # cos(theta)
    phi = 2 * np.pi * np.arange(2 * n) / (2 * n)
    ct, ph = np.meshgrid(x, phi, indexing="ij")
    st = np.sqrt(1 - ct * ct)
    pts = np.stack([st * np.cos(ph), st * np.sin(ph), ct], axis=-1).reshape(-1, 3)
    wts = (w[:, None] * np.full(2 * n, 2 * np.pi / (2 * n))[None, :]).reshape(-1)
    return pts, wts


@pytest.mark.parametrize("l", range(B.MAX_L + 1))
def test_rows_orthonormal_on_sphere(l):
    pts, wts = _sphere_quadrature()
    mono = np.stack([pts[:, 0] ** i * pts[:, 1] ** j * pts[:, 2] ** k for (i, j, k) in B.cart_powers(l)], axis=1)
    Y = mono @ B.solid_harmonic_rows(l).T
    G = (Y * wts[:, None]).T @ Y
    assert np.max(np.abs(G - np.eye(2 * l + 1))) < 1e-12
    # cartesian convention: x^l, y^l, z^l have unit norm
    C = mono @ B.cartesian_rows(l).T
    d = np.einsum("pk,p,pk->k", C, wts, C)
    for idx, p in enumerate(B.cart_powers(l)):
        if max(p) == l:
            assert abs(d[idx] - 1.0) < 1e-12


def test_low_l_conventions():
    """s = 1/sqrt(4 pi); p = (x, y, z) sqrt(3/(4 pi)); d rows xy, yz, 2z^2-x^2-y^2, xz, x^2-y^2."""
    assert np.allclose(B.solid_harmonic_rows(0), [[1 / math.sqrt(4 * math.pi)]], rtol=1e-15)
    assert np.allclose(B.solid_harmonic_rows(1), math.sqrt(3 / (4 * math.pi)) * np.eye(3), rtol=1e-15)
    d = B.solid_harmonic_rows(2)  # monomials xx, xy, xz, yy, yz, zz
    nz = [tuple(np.nonzero(np.abs(r) > 1e-14)[0]) for r in d]
    assert nz == [(1,), (4,), (0, 3, 5), (2,), (0, 3)]
    assert d[2, 5] > 0 and np.isclose(d[2, 0], -0.5 * d[2, 5]) and np.isclose(d[4, 0], -d[4, 3])


@pytest.mark.parametrize("l", [0, 1, 2, 3, 5])
def test_contraction_normalisation(l):
    e = [9.5, 2.1, 0.45, 0.11]
    c = [[0.1, 0.0], [0.4, -0.2], [0.5, 0.7], [0.2, 0.6]]
    a = B.normalized_contraction(l, e, c)
    b = OS.normalise_contraction(l, e, c)
    assert np.max(np.abs(a - b)) < 1e-11 * np.max(np.abs(a))


def _random_shells(seed, max_l=4, cart=False):
    g = np.random.default_rng(seed)
    shells = []
    for l in list(range(max_l + 1)) * 2:
        nprim = int(g.integers(1, 5))
        nctr = int(g.integers(1, 3))
        e = np.sort(np.exp(g.uniform(math.log(0.15), math.log(30.0), nprim)))[::-1]
        c = B.normalized_contraction(l, e, g.uniform(0.1, 1.0, (nprim, nctr)))
        shells.append(B.Shell(g.uniform(-1.5, 1.5, 3), l, e, c))
    return B.ShellBasis(shells, cart=cart)


def _oracle_spec(basis, own_rows=True):
    """The oracle's input: raw shells; own_rows=False hands it the product's rows (for custom rows)."""
    return [(s.centre, s.l, s.exps, s.coefs, None if own_rows and s.rows is None else basis.rows_for(s))
            for s in basis.shells]


def test_whole_ao_norm_and_overlap():
    """int phi_a phi_b d^3r = identity within a spherical shell (one centre, product quadrature)."""
    sh = [B.Shell(np.zeros(3), l, np.array([3.0, 0.7, 0.2]),
                  B.normalized_contraction(l, [3.0, 0.7, 0.2], [[0.3], [0.6], [0.4]])) for l in (0, 1, 2, 3)]
    basis = B.ShellBasis(sh)
    pts, wts = _sphere_quadrature(16)
    xr, wr = np.polynomial.legendre.leggauss(120)
    r = 10.0 * (xr + 1) / 2  # [0, 10] bohr
    wr = wr * 5.0 * r * r
    coords = (r[:, None, None] * pts[None, :, :]).reshape(-1, 3)
    w = (wr[:, None] * wts[None, :]).reshape(-1)
    ao, _, _ = OS.eval_shells(_oracle_spec(basis), coords)
    S = (ao * w[:, None]).T @ ao
    assert np.max(np.abs(S - np.eye(ao.shape[1]))) < 1e-9


@pytest.mark.parametrize("cart", [False, True])
def test_oracle_derivatives_by_finite_differences(cart):
    basis = _random_shells(3, max_l=4, cart=cart)
    spec = _oracle_spec(basis)
    pts = np.random.default_rng(4).uniform(-2, 2, (7, 3))
    ao, g1, g2 = OS.eval_shells(spec, pts, cart=cart)
    h = 1e-4
    for i in range(3):
        dp = np.zeros(3)
        dp[i] = h
        ap, _, _ = OS.eval_shells(spec, pts + dp, cart=cart)
        am, _, _ = OS.eval_shells(spec, pts - dp, cart=cart)
        fd1 = (ap - am) / (2 * h)
        fd2 = (ap - 2 * ao + am) / (h * h)
        assert np.max(np.abs(fd1 - g1[:, :, i])) < 1e-6 * max(1.0, np.max(np.abs(g1)))
        assert np.max(np.abs(fd2 - g2[:, :, i])) < 1e-4 * max(1.0, np.max(np.abs(g2)))


def test_synthetic_basis_through_shells():
    wl = synthetic.make_workload(500, 40, 6, seed=5, box_angstrom=6.0, centre_box_angstrom=3.0)
    sb = B.ShellBasis.from_synthetic(wl.basis)
    assert sb.n_ao == 40
    got = OS.eval_shells(_oracle_spec(sb, own_rows=False), wl.coords)
    ref = O.eval_ao_planes(wl.basis, wl.coords)
    for a, b in zip(got, ref):
        assert np.max(np.abs(a - b)) < 1e-12 * np.max(np.abs(b))


def test_from_libcint_arrays():
    """PySCF's libcint layout: _atm (charge, coord offset, ...), _bas rows, _env doubles."""
    env = [0.0] * 20
    atm = np.zeros((2, 6), dtype=np.int32)
    atm[0, :2] = (8, 20)
    atm[1, :2] = (1, 23)
    env += [0.0, 0.0, 0.2, 1.4, 0.3, -0.1]  # coordinates at 20 and 23
    e_s, c_s = [5.0, 1.0, 0.25], B.normalized_contraction(0, [5.0, 1.0, 0.25], [[0.2, 0.1], [0.5, -0.4], [0.4, 1.0]])
    e_p, c_p = [1.3, 0.3], B.normalized_contraction(1, [1.3, 0.3], [[0.5], [0.6]])
    e_d, c_d = [0.8], B.normalized_contraction(2, [0.8], [[1.0]])
    bas = []
    for ia, l, e, c in ((0, 0, e_s, c_s), (0, 1, e_p, c_p), (1, 2, e_d, c_d)):
        pe = len(env)
        env += list(e)
        pc = len(env)
        env += list(np.asarray(c).T.reshape(-1))
        bas.append([ia, l, len(e), np.asarray(c).shape[1], 0, pe, pc, 0])
    sb = B.ShellBasis.from_libcint(atm, np.asarray(bas, dtype=np.int32), np.asarray(env))
    assert [s.l for s in sb.shells] == [0, 1, 2]
    assert sb.n_ao == 2 + 3 + 5
    assert np.allclose(sb.shells[2].centre, [1.4, 0.3, -0.1])
    assert np.allclose(sb.shells[0].coefs, c_s)
    t = sb.host_tables()
    # l, nprim, exponent offset, coefficient offset, first AO, components, contractions, row offset
    assert t["shell"].tolist() == [[0, 3, 0, 0, 0, 1, 2, 0], [1, 2, 3, 6, 2, 3, 1, 1], [2, 1, 5, 8, 5, 5, 1, 10]]
    # AO order: contraction-major within a shell
    assert t["ao"][:, :3].tolist() == ([[0, 0, 0], [0, 1, 0], [1, 0, 0], [1, 0, 1], [1, 0, 2]]
                                       + [[2, 0, k] for k in range(5)])
    assert t["trans"].size == 1 * 1 + 3 * 3 + 5 * 6
    cart = B.ShellBasis.from_libcint(atm, np.asarray(bas, dtype=np.int32), np.asarray(env), cart=True)
    assert cart.n_ao == 2 + 3 + 6


def test_validate_rejects_bad_shells():
    ok = B.Shell(np.zeros(3), 1, np.array([1.0]), np.array([[1.0]]))
    with pytest.raises(ValueError):
        B.ShellBasis([B.Shell(np.zeros(3), 7, np.array([1.0]), np.array([[1.0]]))]).validate()
    with pytest.raises(ValueError):
        B.ShellBasis([B.Shell(np.zeros(3), 0, np.array([-1.0]), np.array([[1.0]]))]).validate()
    with pytest.raises(ValueError):
        B.ShellBasis([B.Shell(np.zeros(3), 1, np.array([1.0]), np.array([[1.0]]), rows=np.ones((1, 2)))]).validate()
    with pytest.raises(ValueError):
        B.ShellBasis([]).validate()
    B.ShellBasis([ok]).validate()
