"""CPU restatement of contracted Gaussian AO evaluation (test infrastructure only).

The reference takes phi, grad phi and the diagonal second derivatives from
PySCF (``numint.eval_ao``, called at ``interface/pyscf.py:824, 849-852`` and in
``ao_grads``, ``interface/pyscf.py:677-705``; PySCF >= 2.3.0 per the
reference's requirements).  PySCF is not installed here, so this is a
restatement of the published definitions, not a pinned copy:

* a shell of angular momentum l at centre R with primitives (alpha_p) and
  contraction columns C[:, c] gives, for each column and each angular
  component k, phi(r) = sum_p C[p, c] exp(-alpha_p |r-R|^2) A_k(r - R);
* spherical components A_k = r^l Y_lm(r_hat) with real, unit-norm spherical
  harmonics without the Condon-Shortley phase, ordered (x, y, z) for l = 1 and
  m = -l..l otherwise; built here by fitting r^l times SciPy's complex
  harmonics (``scipy.special.sph_harm_y``) on the cartesian monomials;
* cartesian components sqrt((2l+1)/(4 pi)) x^i y^j z^k, i = l..0, j = l-i..0;
* contraction normalisation: each primitive r^l exp(-alpha r^2) scaled to unit
  radial norm, then each column to unit norm of its contracted radial function,
  both by numerical quadrature (scipy.integrate.quad).

Parity against PySCF itself is unpinned; the tests pin these definitions by
properties (orthonormality on the sphere, unit norm of whole AOs, finite
differences) and against the seeded synthetic basis of ``ao_numpy``.
"""
from __future__ import annotations

import math

import numpy as np


def cart_powers(l):
    return [(i, j, l - i - j) for i in range(l, -1, -1) for j in range(l - i, -1, -1)]


def _real_ylm(l, m, theta, phi):
    """Real unit-norm spherical harmonic without the Condon-Shortley phase."""
    from scipy.special import sph_harm_y

    am = abs(m)
    y = sph_harm_y(l, am, theta, phi)  # includes (-1)^m for m > 0
    if m == 0:
        return y.real
    cs = (-1.0) ** am
    return math.sqrt(2.0) * cs * (y.imag if m < 0 else y.real)


def spherical_rows(l, n_fit=400, seed=0):
    """(2l+1, ncart) rows: r^l Y_lm as a combination of x^i y^j z^k (least squares, exact in exact arithmetic)."""
    order = [1, -1, 0] if l == 1 else list(range(-l, l + 1))
    g = np.random.default_rng(seed)
    pts = g.standard_normal((n_fit, 3))
    r = np.linalg.norm(pts, axis=1)
    theta = np.arccos(np.clip(pts[:, 2] / r, -1.0, 1.0))
    phi = np.arctan2(pts[:, 1], pts[:, 0])
    mono = np.stack([pts[:, 0] ** i * pts[:, 1] ** j * pts[:, 2] ** k for (i, j, k) in cart_powers(l)], axis=1)
    rows = []
    for m in order:
        target = r ** l * _real_ylm(l, m, theta, phi)
        coef, *_ = np.linalg.lstsq(mono, target, rcond=None)
        coef[np.abs(coef) < 1e-12 * np.max(np.abs(coef))] = 0.0
        rows.append(coef)
    return np.asarray(rows)


def cartesian_rows(l):
    return math.sqrt((2 * l + 1) / (4.0 * math.pi)) * np.eye((l + 1) * (l + 2) // 2)


def normalise_contraction(l, exps, coefs):
    """(nprim, nctr) basis-file coefficients -> unit-norm contracted radial functions (quadrature)."""
    from scipy.integrate import quad

    e = np.asarray(exps, dtype=np.float64)
    c = np.array(coefs, dtype=np.float64).reshape(e.size, -1)
    for p in range(e.size):
        n2, _ = quad(lambda r: r ** (2 * l + 2) * math.exp(-2.0 * e[p] * r * r), 0.0, np.inf, epsabs=0, epsrel=1e-13)
        c[p] /= math.sqrt(n2)
    for k in range(c.shape[1]):
        def f(r, k=k):
            return (r ** l * np.sum(c[:, k] * np.exp(-e * r * r))) ** 2 * r * r
        n2, _ = quad(f, 0.0, np.inf, epsabs=0, epsrel=1e-13, limit=200)
        c[:, k] /= math.sqrt(n2)
    return c


def eval_shells(shells, coords, cart=False):
    """ao (N, n_ao), grad (N, n_ao, 3), diagonal second derivatives (N, n_ao, 3).

    ``shells``: sequence of (centre (3,), l, exps (nprim,), coefs (nprim, nctr),
    rows (ncomp, ncart) or None for the spherical/cartesian convention).
    """
    coords = np.asarray(coords, dtype=np.float64)
    cols_v, cols_g, cols_h = [], [], []
    for centre, l, exps, coefs, rows in shells:
        l = int(l)
        if rows is None:
            rows = cartesian_rows(l) if cart else spherical_rows(l)
        rows = np.asarray(rows, dtype=np.float64)
        e = np.asarray(exps, dtype=np.float64)
        c = np.asarray(coefs, dtype=np.float64).reshape(e.size, -1)
        d = coords - np.asarray(centre, dtype=np.float64)[None, :]
        r2 = np.sum(d * d, axis=1)
        ex = np.exp(-r2[:, None] * e[None, :])  # (N, nprim)
        # radial g(r2) and its derivatives with respect to each coordinate
        g = ex @ c  # (N, nctr)
        gp = (ex * (-2.0 * e)[None, :]) @ c  # d g / d x_i = x_i * gp
        gpp = (ex * (4.0 * e * e)[None, :]) @ c
        pw = cart_powers(l)
        mono = np.empty((coords.shape[0], len(pw)))
        dmono = np.empty((3, coords.shape[0], len(pw)))
        d2mono = np.empty((3, coords.shape[0], len(pw)))
        for q, p in enumerate(pw):
            mono[:, q] = np.prod([d[:, i] ** p[i] for i in range(3)], axis=0)
            for i in range(3):
                pi = list(p)
                f1 = pi[i]
                pi[i] = max(pi[i] - 1, 0)
                dmono[i, :, q] = f1 * np.prod([d[:, k] ** pi[k] for k in range(3)], axis=0) if f1 else 0.0
                pj = list(p)
                f2 = p[i] * (p[i] - 1)
                pj[i] = max(p[i] - 2, 0)
                d2mono[i, :, q] = f2 * np.prod([d[:, k] ** pj[k] for k in range(3)], axis=0) if f2 else 0.0
        A = mono @ rows.T  # (N, ncomp)
        dA = np.einsum("inq,kq->ink", dmono, rows)
        d2A = np.einsum("inq,kq->ink", d2mono, rows)
        for k in range(c.shape[1]):
            gk, gpk, gppk = g[:, k:k + 1], gp[:, k:k + 1], gpp[:, k:k + 1]
            cols_v.append(A * gk)
            gr = np.stack([dA[i] * gk + A * d[:, i:i + 1] * gpk for i in range(3)], axis=-1)
            he = np.stack([d2A[i] * gk + 2.0 * dA[i] * d[:, i:i + 1] * gpk
                           + A * (gpk + d[:, i:i + 1] ** 2 * gppk) for i in range(3)], axis=-1)
            cols_g.append(gr)
            cols_h.append(he)
    return np.concatenate(cols_v, axis=1), np.concatenate(cols_g, axis=1), np.concatenate(cols_h, axis=1)
