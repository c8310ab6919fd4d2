"""CPU restatement of the nu integrals and the chi tensor (test infrastructure only).

nu_ab(C) = int phi_a(r) phi_b(r) erf(omega |r - C|) / |r - C| dr (omega = 0:
1/|r - C|) is what the reference obtains from PySCF's int1e_grids
(external/_hf_density.py:17-120, PySCF >= 2.3.0, not installed here), and

    chi[r, w, s, a] = sum_(b,d) D_s[b, d] phi_b(r) nu^(omega_w)_(d a)(r)

is generate_chi_tensor (interface/pyscf.py:1067-1126).  The integrals are the
McMurchie-Davidson scheme (Helgaker, Jorgensen, Olsen, Molecular
Electronic-Structure Theory, ch. 9): Hermite expansion coefficients of the
Gaussian product, Hermite Coulomb integrals R_tuv from the Boys function, and
the attenuated operator as the Coulomb potential of a Gaussian charge of
exponent omega^2 (product exponent p -> mu = p omega^2 / (p + omega^2), overall
factor sqrt(mu / p)).  The Boys function is taken from SciPy's regularised
incomplete gamma function (series for T < 1).  Parity against PySCF is
unpinned; the tests pin these integrals by direct quadrature and by the closed
form of s-type pairs.
"""
from __future__ import annotations

import math

import numpy as np
from scipy.special import gamma, gammainc

from .shells import cart_powers, cartesian_rows, spherical_rows


def boys(nmax: int, T) -> np.ndarray:
    """F_n(T) = int_0^1 u^(2n) exp(-T u^2) du for n = 0..nmax; shape (nmax + 1,) + T.shape."""
    T = np.asarray(T, dtype=np.float64)
    out = np.empty((nmax + 1,) + T.shape)
    small = T < 1.0
    Ts, Tl = T[small], T[~small]
    for n in range(nmax + 1):
        term = np.full(Ts.shape, 1.0 / (2 * n + 1))
        s = term.copy()
        for k in range(1, 40):
            term = term * 2.0 * Ts / (2 * n + 2 * k + 1)
            s = s + term
        out[n][small] = np.exp(-Ts) * s
        out[n][~small] = 0.5 * gamma(n + 0.5) * gammainc(n + 0.5, Tl) / Tl ** (n + 0.5)
    return out


def hermite_e(la: int, lb: int, a: float, b: float, xa: float, xb: float) -> np.ndarray:
    """E[i, j, t] of the 1D Gaussian product, i <= la, j <= lb, t <= la + lb."""
    p = a + b
    xp = (a * xa + b * xb) / p
    E = np.zeros((la + 1, lb + 1, la + lb + 2))
    E[0, 0, 0] = math.exp(-a * b / p * (xa - xb) ** 2)
    for i in range(la + 1):
        for j in range(lb + 1):
            if i == 0 and j == 0:
                continue
            if i > 0:
                prev, x = E[i - 1, j], xp - xa
            else:
                prev, x = E[i, j - 1], xp - xb
            for t in range(i + j + 1):
                v = x * prev[t] + (t + 1) * prev[t + 1]
                if t > 0:
                    v += prev[t - 1] / (2 * p)
                E[i, j, t] = v
    return E


def hermite_r(L: int, mu: float, pc: np.ndarray, F: np.ndarray) -> dict:
    """R^0_tuv(mu, P - C) for t + u + v <= L; pc (N, 3), F (L + 1, N)."""
    nxt = {(0, 0, 0): (-2.0 * mu) ** L * F[L]}
    for n in range(L - 1, -1, -1):
        cur = {}
        for t in range(L - n + 1):
            for u in range(L - n + 1 - t):
                for v in range(L - n + 1 - t - u):
                    if t > 0:
                        val = pc[:, 0] * nxt[(t - 1, u, v)]
                        if t > 1:
                            val = val + (t - 1) * nxt[(t - 2, u, v)]
                    elif u > 0:
                        val = pc[:, 1] * nxt[(0, u - 1, v)]
                        if u > 1:
                            val = val + (u - 1) * nxt[(0, u - 2, v)]
                    elif v > 0:
                        val = pc[:, 2] * nxt[(0, 0, v - 1)]
                        if v > 1:
                            val = val + (v - 1) * nxt[(0, 0, v - 2)]
                    else:
                        val = (-2.0 * mu) ** n * F[n]
                    cur[(t, u, v)] = val
        nxt = cur
    return nxt


def nu_primitive(la, lb, a, b, A, B, C, omega) -> np.ndarray:
    """Cartesian primitive block (ncart(la), ncart(lb), N) at points C (N, 3)."""
    A, B, C = np.asarray(A, float), np.asarray(B, float), np.asarray(C, float)
    p = a + b
    P = (a * A + b * B) / p
    mu = p if omega == 0 else p * omega * omega / (p + omega * omega)
    pref = 2.0 * math.pi / p * math.sqrt(mu / p)
    E = [hermite_e(la, lb, a, b, A[d], B[d]) for d in range(3)]
    pc = P[None, :] - C
    L = la + lb
    F = boys(L, mu * np.sum(pc * pc, axis=1))
    R = hermite_r(L, mu, pc, F)
    pa, pb = cart_powers(la), cart_powers(lb)
    out = np.zeros((len(pa), len(pb), C.shape[0]))
    for qa, (i1, k1, m1) in enumerate(pa):
        for qb, (i2, k2, m2) in enumerate(pb):
            s = 0.0
            for t in range(i1 + i2 + 1):
                for u in range(k1 + k2 + 1):
                    for v in range(m1 + m2 + 1):
                        s = s + E[0][i1, i2, t] * E[1][k1, k2, u] * E[2][m1, m2, v] * R[(t, u, v)]
            out[qa, qb] = s
    return pref * out


def nu_integrals(shells, coords, omega: float, cart: bool = False) -> np.ndarray:
    """(N, n_ao, n_ao); shells as for oracle.shells.eval_shells."""
    coords = np.asarray(coords, dtype=np.float64)
    blocks = []
    for centre, l, exps, coefs, rows in shells:
        l = int(l)
        rows = (cartesian_rows(l) if cart else spherical_rows(l)) if rows is None else np.asarray(rows, float)
        c = np.asarray(coefs, float).reshape(len(exps), -1)
        blocks.append((np.asarray(centre, float), l, np.asarray(exps, float), c, rows))
    sizes = [b[3].shape[1] * b[4].shape[0] for b in blocks]
    offs = np.concatenate([[0], np.cumsum(sizes)])
    n = int(offs[-1])
    nu = np.zeros((coords.shape[0], n, n))
    for i, (A, la, ea, ca, ra) in enumerate(blocks):
        for j, (B, lb, eb, cb, rb) in enumerate(blocks):
            if j > i:
                continue
            acc = np.zeros((ca.shape[1], cb.shape[1], ra.shape[1], rb.shape[1], coords.shape[0]))
            for p1, a in enumerate(ea):
                for p2, b in enumerate(eb):
                    prim = nu_primitive(la, lb, a, b, A, B, coords, omega)
                    acc += ca[p1][:, None, None, None, None] * cb[p2][None, :, None, None, None] * prim[None, None]
            # angular rows on both sides: (ctr_a, comp_a, ctr_b, comp_b, N)
            blk = np.einsum("ka,xyabn,lb->xkyln", ra, acc, rb)
            blk = blk.reshape(ca.shape[1] * ra.shape[0], cb.shape[1] * rb.shape[0], -1).transpose(2, 0, 1)
            if i == j:  # a shell with itself: the lower triangle, mirrored
                low = np.tril(np.ones(blk.shape[1:], dtype=bool))
                blk = np.where(low[None], blk, blk.transpose(0, 2, 1))
            nu[:, offs[i]:offs[i + 1], offs[j]:offs[j + 1]] = blk
            nu[:, offs[j]:offs[j + 1], offs[i]:offs[i + 1]] = blk.transpose(0, 2, 1)
    return nu


def generate_chi(rdm1, ao, nus) -> np.ndarray:
    """chi (N, n_omega, 2, n) from the integrals of each omega (interface/pyscf.py:1109-1126)."""
    return np.stack([np.einsum("sbd,rb,rda->rsa", rdm1, ao, nu) for nu in nus], axis=1)
