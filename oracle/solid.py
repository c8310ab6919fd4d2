"""CPU restatement of the k-point (Solid) XC path (test infrastructure only).

Follows solid.py:272-632 (densities as unconjugated bilinear forms summed over
k-points with the KPointInfo weights, one-body and Coulomb energies, the
Coulomb potential) and train.py:86-163 with a Solid (jax.grad of E_xc with
respect to the complex rdm1, F = h1e + J + n_kpt * dE_xc/dD, abs_clip,
(F + F^H)/2, abs_clip).  torch autograd stands in for jax.grad; for a complex
leaf JAX returns dE/dRe - i dE/dIm, the conjugate of torch's gradient.
"""
from __future__ import annotations

import numpy as np
import torch

from .oracle import CLIP, FUNCTIONALS, energy_densities, xc_energy

C128 = torch.complex128


def _c(x) -> torch.Tensor:
    return torch.as_tensor(np.asarray(x)).to(C128)


def _w(x) -> torch.Tensor:
    return torch.as_tensor(np.asarray(x), dtype=torch.float64).to(C128)


def cabs_clip(x, thr):
    return torch.where(x.abs() > thr, x, torch.zeros((), dtype=x.dtype))


def solid_features(rdm1, ao, grad_ao, grad2_ao, kweights):
    """rho (grid, 2), grad rho (grid, 2, 3), lapl (grid, 2), tau (grid, 2): solid.py:491-632."""
    D, a, g = (rdm1 if isinstance(rdm1, torch.Tensor) else _c(rdm1)), _c(ao), _c(grad_ao)
    w = _w(kweights)
    rho = torch.einsum("k,skab,kra,krb->rs", w, D, a, a).real
    grad = 2 * torch.einsum("k,skab,kra,krbj->rsj", w, D, a, g).real
    gg = torch.einsum("k,skab,kraj,krbj->rs", w, D, g, g)
    lapl = None
    if grad2_ao is not None:
        lapl = (2 * gg + 2 * torch.einsum("k,skab,kra,krbi->rs", w, D, a, _c(grad2_ao))).real
    tau = 0.5 * gg.real
    return rho, grad, lapl, tau


def solid_xc_energy_and_grads(name, rdm1, ao, grad_ao, grad2_ao, weights, kweights, clip_cte=CLIP):
    """(E_xc, jax.grad of E_xc with respect to the complex rdm1)."""
    D = _c(rdm1).clone().requires_grad_(True)
    rho, grad, lapl, tau = solid_features(D, ao, grad_ao, grad2_ao, kweights)
    dens = energy_densities(name, rho, grad, lapl, tau, None, clip_cte)
    _, coeffs = FUNCTIONALS[name]
    E = xc_energy(torch.tensor([coeffs], dtype=torch.float64), dens, torch.as_tensor(np.asarray(weights)), clip_cte)
    (g,) = torch.autograd.grad(E, [D])
    return float(E.detach()), g.conj().resolve_conj().detach().numpy()


def solid_coulomb(rep, rdm1, kweights):
    """solid.py:302-330: v[k] = w_k sum rep[k,q,i,j,l,m] D_q[m,l] with D summed over spin."""
    return torch.einsum("k,kqijlm,qml->kij", _w(kweights), _c(rep), _c(rdm1).sum(0)).numpy()


def solid_nonxc(rdm1, h1e, rep, nuclear_repulsion, kweights):
    """solid.py:272-411."""
    D, w = _c(rdm1).sum(0), _w(kweights)
    one = torch.einsum("k,kij,kji->", w, D, _c(h1e)).real
    v = torch.as_tensor(solid_coulomb(rep, rdm1, kweights))
    coul = (torch.einsum("k,kij,kji->", w, D, v) / 2.0).real
    return float(nuclear_repulsion + one + coul)


def solid_predict(name, rdm1, ao, grad_ao, grad2_ao, weights, kweights, h1e, rep, nuclear_repulsion,
                  clip_cte=CLIP):
    """train.py:124-163 with a Solid: (E, F)."""
    exc, vxc = solid_xc_energy_and_grads(name, rdm1, ao, grad_ao, grad2_ao, weights, kweights, clip_cte)
    K = np.asarray(rdm1).shape[1]
    F = _c(h1e) + torch.as_tensor(solid_coulomb(rep, rdm1, kweights)) + torch.as_tensor(vxc) * K
    F = cabs_clip(F, clip_cte)
    F = 0.5 * (F + F.transpose(-1, -2).conj().resolve_conj())
    F = cabs_clip(F, clip_cte)
    return exc + solid_nonxc(rdm1, h1e, rep, nuclear_repulsion, kweights), F.numpy()
