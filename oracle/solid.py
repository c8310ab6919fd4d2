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


def solid_fock_solver(fock, s1e):
    """safe_fock_solver (utils/eigenproblem.py:110-149) on k-point batches, as the reference runs it for
    a Solid: C = L^-1 F L^-T (no conjugation) with B = L L^H, eigh of its lower triangle, L^-T C'."""
    L = torch.linalg.cholesky(_c(s1e))
    L_inv = torch.linalg.inv(L)
    out_e, out_c = [], []
    for s in range(2):
        C = L_inv @ _c(fock[s]) @ L_inv.transpose(-1, -2)
        e, v = torch.linalg.eigh(C)
        out_e.append(e)
        out_c.append(L_inv.transpose(-1, -2) @ v)
    return torch.stack(out_e), torch.stack(out_c)


def solid_get_occ(mo_energy, nelecs):
    """solid.py:438-487: per spin and k-point, the nelec lowest orbitals."""
    occ = torch.zeros(mo_energy.shape, dtype=torch.float64)
    for s in range(2):
        for k in range(mo_energy.shape[1]):
            idx = torch.argsort(mo_energy[s, k])
            occ[s, k, idx[:int(nelecs[s])]] = 1.0
    return occ


def solid_make_rdm1(mo_coeff, mo_occ):
    """solid.py:413-435."""
    return torch.einsum("skij,skj,sklj->skil", mo_coeff, mo_occ.to(C128), mo_coeff.conj())


def solid_scf_loop(name, rdm1, mo_occ, ao, grad_ao, grad2_ao, weights, kweights, h1e, s1e, rep, nuclear_repulsion,
                   cycles, mixing_factor=0.4, clip_cte=CLIP):
    """diff_simple_scf_loop (evaluate.py:256-344) with a Solid: (energy, rdm1, fock, mo_energy)."""
    nelecs = [int(round(float(np.asarray(mo_occ)[s, 0].sum()))) for s in range(2)]
    D = _c(rdm1)
    E, F = solid_predict(name, D.numpy(), ao, grad_ao, grad2_ao, weights, kweights, h1e, rep, nuclear_repulsion,
                         clip_cte)
    mo_e = None
    for _ in range(cycles):
        mo_e, mo_c = solid_fock_solver(F, s1e)
        occ = solid_get_occ(mo_e, nelecs)
        D = (1 - mixing_factor) * D + mixing_factor * solid_make_rdm1(mo_c, occ)
        E, F = solid_predict(name, D.resolve_conj().numpy(), ao, grad_ao, grad2_ao, weights, kweights, h1e, rep,
                             nuclear_repulsion, clip_cte)
    return E, D.resolve_conj().numpy(), F, mo_e.numpy()
