"""Oracle for the differentiable SCF loop (test infrastructure, CPU, FP64).

A CPU restatement of ``diff_simple_scf_loop`` (evaluate.py:256-344) on the
oracle's own XC energy (oracle.py), differentiated end to end by torch
autograd: V_xc = dE_xc/dD is formed with ``create_graph=True`` so the outer
gradient differentiates through it, as jax.grad does in the reference.  The
eigensolver follows utils/eigenproblem.py:26-149 (Cholesky reduction and the
Lorentzian-broadened reverse rule), occupations molecule.py:848-889, the
Fock matrix train.py:147-163.  Only tests may import this module.
"""
from __future__ import annotations

import torch

from .oracle import CLIP, _energy, _tree_leaves, abs_clip, t64

DEGEN_TOL = 1e-6
BROADENING = 1e-10


class _Eigh(torch.autograd.Function):
    @staticmethod
    def forward(ctx, A):
        e, v = torch.linalg.eigh(A)
        ctx.save_for_backward(e, v)
        return e, v

    @staticmethod
    def backward(ctx, ge, gv):
        e, v = ctx.saved_tensors
        ge = torch.zeros_like(e) if ge is None else ge
        gv = torch.zeros_like(v) if gv is None else gv
        vt = v.T
        diff = e.reshape(1, -1) - e.reshape(-1, 1)
        non = (diff.abs() >= DEGEN_TOL).to(e.dtype)
        deg = (diff.abs() < DEGEN_TOL).to(e.dtype)
        with torch.no_grad():
            reg = torch.nan_to_num(1.0 / diff)
        F = 0.5 * (non * reg + deg * (diff / (diff * diff + BROADENING)))
        F = F - torch.diag(torch.diag(F))
        grad = torch.linalg.inv(vt) @ (0.5 * torch.diag(ge) + F * (vt @ gv)) @ vt
        return grad + grad.T


def _general_eigh(A, B):
    L_inv = torch.linalg.inv(torch.linalg.cholesky(B))
    e, v = _Eigh.apply(L_inv @ A @ L_inv.T)
    return e, L_inv.T @ v


def scf_energy_and_grads(params, ao, grad_ao, grad2_ao, weights, ehf, h1e, s1e, df_tensor, nuclear_repulsion,
                         rdm1, mo_occ, cycles, mixing_factor, name="DM21", clip_cte=CLIP):
    """Final energy of the unrolled loop and its gradient with respect to the parameters."""
    ao, grad_ao, grad2_ao, weights = t64(ao), t64(grad_ao), t64(grad2_ao), t64(weights)
    ehf, h1e, s1e, df = t64(ehf), t64(h1e), t64(s1e), t64(df_tensor)
    p, names = _tree_leaves(params)
    tp = {"params": {k: {} for k in p}}
    leaves = []
    for k, kk in names:
        t = t64(p[k][kk]).clone().requires_grad_(True)
        tp["params"][k][kk] = t
        leaves.append(((k, kk), t))
    nelec = [int(round(float(t64(mo_occ)[s].sum()))) for s in range(2)]

    def energy_fock(D):
        Dl = D if D.requires_grad else D.clone().requires_grad_(True)
        exc = _energy(name, Dl, ao, grad_ao, grad2_ao, weights, tp, ehf, clip_cte)
        (vxc,) = torch.autograd.grad(exc, Dl, create_graph=True)
        dt = D.sum(0)
        J = torch.einsum("P,Pmn->mn", torch.einsum("Pls,ls->P", df, dt), df)
        e = exc + float(nuclear_repulsion) + torch.sum(dt * h1e) + 0.5 * torch.sum(dt * J)
        f = abs_clip(h1e + J + vxc, clip_cte)
        f = 0.5 * (f + f.transpose(-1, -2))
        return e, abs_clip(f, clip_cte)

    D = t64(rdm1)
    e, fock = energy_fock(D)
    for _ in range(cycles):
        es, cs = zip(*[_general_eigh(fock[s], s1e) for s in range(2)])
        occ = torch.zeros(2, D.shape[-1], dtype=D.dtype)
        for s in range(2):
            occ[s, torch.argsort(es[s].detach())[: nelec[s]]] = 1.0
        C = torch.stack(cs)
        D = (1.0 - mixing_factor) * D + mixing_factor * torch.einsum("sij,sj,skj->sik", C, occ, C)
        e, fock = energy_fock(D)
    grads = torch.autograd.grad(e, [t for _, t in leaves])
    out = {}
    for ((k, kk), _), g in zip(leaves, grads):
        out.setdefault(k, {})[kk] = g.detach().numpy()
    return float(e.detach()), {"params": out}, D.detach().numpy()
