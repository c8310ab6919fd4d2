"""Oracle AO evaluation (numpy, float64) for the synthetic Gaussian basis.

Test infrastructure only.  It stands in for PySCF's ``numint.eval_ao`` with
``deriv=1`` plus the diagonal second derivatives of ``ao_grads(order=2)``
(``interface/pyscf.py:677-705, 849-852``) on the seeded basis of
``graddft_gb300.synthetic``.

For ``phi = N P(x,y,z) exp(-alpha r^2)`` (r relative to the centre):
``d_i phi = N (d_i P - 2 alpha x_i P) e`` and
``d_i^2 phi = N (d_i^2 P - 2 alpha P - 4 alpha x_i d_i P + 4 alpha^2 x_i^2 P) e``.
"""
from __future__ import annotations

import numpy as np


def _poly(kind, comp, x, y, z):
    """P, dP/dx_i (3), d2P/dx_i^2 (3) for every (grid, ao) pair."""
    one = np.ones_like(x)
    zero = np.zeros_like(x)
    P = np.empty_like(x)
    dP = np.empty((3,) + x.shape)
    d2P = np.zeros((3,) + x.shape)
    # s
    m = kind == 0
    P[:, m] = 1.0
    dP[:, :, m] = 0.0
    # p
    for c, v in enumerate((x, y, z)):
        m = (kind == 1) & (comp == c)
        P[:, m] = v[:, m]
        for i in range(3):
            dP[i][:, m] = (one if i == c else zero)[:, m]
    # d: xy, yz, xz
    pairs = {0: (0, 1), 1: (1, 2), 2: (0, 2)}
    xyz = (x, y, z)
    for c, (i0, i1) in pairs.items():
        m = (kind == 2) & (comp == c)
        P[:, m] = (xyz[i0] * xyz[i1])[:, m]
        for i in range(3):
            if i == i0:
                dP[i][:, m] = xyz[i1][:, m]
            elif i == i1:
                dP[i][:, m] = xyz[i0][:, m]
            else:
                dP[i][:, m] = 0.0
    # x^2 - y^2
    m = (kind == 2) & (comp == 3)
    P[:, m] = (x * x - y * y)[:, m]
    dP[0][:, m] = (2 * x)[:, m]
    dP[1][:, m] = (-2 * y)[:, m]
    dP[2][:, m] = 0.0
    d2P[0][:, m] = 2.0
    d2P[1][:, m] = -2.0
    # 2z^2 - x^2 - y^2
    m = (kind == 2) & (comp == 4)
    P[:, m] = (2 * z * z - x * x - y * y)[:, m]
    dP[0][:, m] = (-2 * x)[:, m]
    dP[1][:, m] = (-2 * y)[:, m]
    dP[2][:, m] = (4 * z)[:, m]
    d2P[0][:, m] = -2.0
    d2P[1][:, m] = -2.0
    d2P[2][:, m] = 4.0
    return P, dP, d2P


def eval_ao_planes(basis, coords: np.ndarray, chunk: int = 8192):
    """Return ao (N,n), grad_ao (N,n,3), grad2_ao (N,n,3) (diagonal second derivatives)."""
    coords = np.asarray(coords, dtype=np.float64)
    n_grid = coords.shape[0]
    n = basis.n_ao
    ao = np.empty((n_grid, n))
    g1 = np.empty((n_grid, n, 3))
    g2 = np.empty((n_grid, n, 3))
    alpha = basis.exponents[None, :]
    for s in range(0, n_grid, chunk):
        e = min(n_grid, s + chunk)
        d = coords[s:e, None, :] - basis.centres[None, :, :]
        x, y, z = d[..., 0], d[..., 1], d[..., 2]
        r2 = x * x + y * y + z * z
        ex = basis.norm[None, :] * np.exp(-alpha * r2)
        P, dP, d2P = _poly(basis.kind, basis.comp, x, y, z)
        ao[s:e] = P * ex
        for i, xi in enumerate((x, y, z)):
            g1[s:e, :, i] = (dP[i] - 2 * alpha * xi * P) * ex
            g2[s:e, :, i] = (d2P[i] - 2 * alpha * P - 4 * alpha * xi * dP[i] + 4 * alpha * alpha * xi * xi * P) * ex
    return ao, g1, g2
