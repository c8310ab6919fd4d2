"""Differentiable SCF loops on the GPU (evaluate.py:256-344 and 917-1210) with the safe eigensolver.

``diff_simple_scf_loop``: an initial energy/Fock evaluation, then ``cycles``
iterations of generalized eigh of the Fock matrix, aufbau occupations, the
density matrix, linear mixing and a new energy/Fock evaluation.
``diff_scf_loop``: the same with the Fock matrix extrapolated by CDIIS
(``JittableDiis``) instead of density mixing.  Both are differentiable end to
end.  The pieces follow the reference:

* ``safe_eigh`` / ``safe_general_eigh`` / ``safe_fock_solver``:
  utils/eigenproblem.py:26-149, including the Lorentzian-broadened reverse rule
  for (near-)degenerate eigenvalues (DEGEN_TOL 1e-6, BROADENING 1e-10);
* ``get_occ`` / ``make_rdm1``: molecule.py:816-889;
* the energy and Fock matrix of ``energy_predictor.predict``
  (train.py:124-163): E = E_xc + E_nuc + tr(D h) + 1/2 tr(D J) and
  F = abs_clip(1/2 (G + G^T)), G = abs_clip(h + J + V_xc).

The n x n linear algebra (Cholesky, inverse, eigh) runs in FP64 through
torch's CUDA linear-algebra calls (cuSOLVER/cuBLAS); E_xc and V_xc come from
the library's kernels, and the backward through V_xc uses its
Hessian-vector product (one recomputation of the network pass per iteration:
per-iteration checkpointing).  The Coulomb matrix comes from the molecule's
four-index ``rep_tensor`` or, for larger bases, a three-index
density-fitting tensor ``df_tensor`` (naux, n, n): J = sum_P B_P tr(B_P D).
"""
from __future__ import annotations

from typing import Callable

import torch

from . import engine
from .functional import CLIP

DEGEN_TOL = 1e-6
BROADENING = 1e-10
F64 = torch.float64


# The linear algebra of the SCF loop runs without torch's error checks: each
# check copies the solver's info code to the host, a synchronisation per call
# that left the GPU idle between the iterations' kernels (about 180 per
# 20-cycle loop).  JAX's solvers, which the reference uses, do not check
# either: a failed factorisation gives NaN, not an exception.
def _eigh(A):
    op = getattr(torch, "_linalg_eigh", None)  # torch.linalg.eigh without its info check
    return op(A, "L", True) if op is not None else torch.linalg.eigh(A)


def _inv(A):
    return torch.linalg.inv_ex(A).inverse


def _cholesky(A):
    return torch.linalg.cholesky_ex(A).L


class _SafeEigh(torch.autograd.Function):
    """eigh with the reverse rule of utils/eigenproblem.py:41-107."""

    @staticmethod
    def forward(ctx, A):
        evals, evecs = _eigh(A)
        ctx.save_for_backward(evals, evecs)
        return evals, evecs

    @staticmethod
    def backward(ctx, g_evals, g_evecs):
        evals, evecs = ctx.saved_tensors
        if g_evals is None:
            g_evals = torch.zeros_like(evals)
        if g_evecs is None:
            g_evecs = torch.zeros_like(evecs)
        vt = evecs.transpose(-1, -2)
        diff = evals.unsqueeze(-2) - evals.unsqueeze(-1)  # [i][j] = e_j - e_i
        degen = diff.abs() < DEGEN_TOL
        regular = torch.nan_to_num(1.0 / diff, nan=0.0, posinf=torch.finfo(F64).max, neginf=-torch.finfo(F64).max)
        broadened = diff / (diff * diff + BROADENING)
        Fm = 0.5 * torch.where(degen, broadened, regular)
        Fm = Fm - torch.diag_embed(torch.diagonal(Fm, dim1=-2, dim2=-1))
        inner = 0.5 * torch.diag_embed(g_evals) + Fm * (vt @ g_evecs)
        grad = _inv(vt) @ inner @ vt
        return grad + grad.transpose(-1, -2)


def safe_eigh(A):
    """Eigenvalues and eigenvectors of a real symmetric matrix (eigenproblem.py:26-38)."""
    return _SafeEigh.apply(A)


def safe_general_eigh(A, B):
    """A C = B C E via Cholesky of B (eigenproblem.py:110-131)."""
    L = _cholesky(B)
    L_inv = _inv(L)
    C = L_inv @ A @ L_inv.transpose(-1, -2)
    evals, evecs_t = safe_eigh(C)
    return evals, L_inv.transpose(-1, -2) @ evecs_t


def safe_fock_solver(fock, overlap):
    """Both spins (eigenproblem.py:134-149): (mo_energy (2, n), mo_coeff (2, n, n))."""
    e_up, c_up = safe_general_eigh(fock[0], overlap)
    e_dn, c_dn = safe_general_eigh(fock[1], overlap)
    return torch.stack((e_up, e_dn)), torch.stack((c_up, c_dn))


def get_occ(mo_energies, nelecs):
    """Aufbau occupations: the nelec lowest orbitals of each spin (molecule.py:848-889)."""
    occ = torch.zeros_like(mo_energies)
    for s in range(2):
        idx = torch.argsort(mo_energies[s].detach())
        occ[s, idx[: int(nelecs[s])]] = 1.0
    return occ


def make_rdm1(mo_coeff, mo_occ):
    """D_s = C_s diag(occ_s) C_s^T (molecule.py:816-846)."""
    return torch.einsum("sij,sj,skj->sik", mo_coeff, mo_occ, mo_coeff)


def _abs_clip(x, clip):
    return torch.where(x.abs() > clip, x, torch.zeros((), dtype=x.dtype, device=x.device))


def coulomb_matrix(atoms, rdm1_total):
    """J from rep_tensor (molecule.py:783-811) or from a density-fitting tensor."""
    df = getattr(atoms, "df_tensor", None)
    if df is not None:
        return torch.einsum("P,Pmn->mn", torch.einsum("Pls,ls->P", df, rdm1_total), df)
    if atoms.rep_tensor is None:
        raise ValueError("the molecule has neither rep_tensor nor df_tensor for the Coulomb matrix")
    return torch.einsum("mnls,ls->mn", atoms.rep_tensor, rdm1_total)


def energy_and_fock(functional, params, atoms, clip_cte: float = CLIP):
    """energy_predictor.predict (train.py:124-163), differentiable in rdm1 and params (also through V_xc)."""
    exc, vxc = functional.xc_energy_and_potential(params, atoms, clip_cte)
    rdm1 = atoms.rdm1
    d_tot = rdm1.sum(0)
    h1e = atoms.h1e
    J = coulomb_matrix(atoms, d_tot)
    energy = exc + atoms.nuclear_repulsion + torch.sum(d_tot * h1e) + 0.5 * torch.sum(d_tot * J)
    fock = _abs_clip(h1e + J + vxc, clip_cte)
    fock = 0.5 * (fock + fock.transpose(-1, -2))
    return energy, _abs_clip(fock, clip_cte)


def _to_device(atoms):
    dev = atoms.resident().device
    t = lambda x: x if isinstance(x, torch.Tensor) and x.device == dev else torch.as_tensor(x, dtype=F64, device=dev)  # noqa: E731
    atoms = atoms.replace(rdm1=t(atoms.rdm1), h1e=t(atoms.h1e), s1e=t(atoms.s1e),
                          nuclear_repulsion=t(atoms.nuclear_repulsion), mo_occ=t(atoms.mo_occ))
    if getattr(atoms, "df_tensor", None) is not None:
        return atoms.replace(df_tensor=t(atoms.df_tensor))
    if atoms.rep_tensor is not None:
        return atoms.replace(rep_tensor=t(atoms.rep_tensor))
    return atoms


# ---------------------------------------------------------------- solids
def solid_fock_solver(fock, s1e):
    """safe_fock_solver (utils/eigenproblem.py:110-149) as the reference applies it to a Solid's
    k-point batches: B = L L^H, C = L^-1 F L^-T (no conjugation), eigh of C's lower triangle,
    eigenvectors L^-T C'.  fock (2, n_kpt, n, n), s1e (n_kpt, n, n): (mo_energy, mo_coeff)."""
    L_inv = torch.linalg.inv(torch.linalg.cholesky(s1e))
    es, cs = [], []
    for s in range(2):
        e, v = torch.linalg.eigh(L_inv @ fock[s] @ L_inv.transpose(-1, -2))
        es.append(e)
        cs.append(L_inv.transpose(-1, -2) @ v)
    return torch.stack(es), torch.stack(cs)


def solid_get_occ(mo_energy, nelecs):
    """solid.py:438-487: the nelec lowest orbitals of each spin and k-point."""
    occ = torch.zeros(mo_energy.shape, dtype=F64, device=mo_energy.device)
    idx = torch.argsort(mo_energy, dim=-1)
    for s in range(2):
        occ[s].scatter_(-1, idx[s, :, :int(nelecs[s])], 1.0)
    return occ


def solid_make_rdm1(mo_coeff, mo_occ):
    """solid.py:413-435: D[s,k] = C diag(occ) C^H."""
    return torch.einsum("skij,skj,sklj->skil", mo_coeff, mo_occ.to(mo_coeff.dtype), mo_coeff.conj())


def _solid_scf(functional, params, atoms, cycles, mixing_factor, clip_cte):
    """diff_simple_scf_loop (evaluate.py:256-344) with a Solid: linear mixing around the k-point predict.
    With constant-coefficient functionals nothing depends on parameters, so the loop runs forward."""
    from .train import energy_predictor

    predict = energy_predictor(functional, clip_cte=clip_cte)
    dev = atoms.device
    c = lambda x: torch.as_tensor(x).to(device=dev, dtype=torch.complex128)  # noqa: E731
    atoms = atoms.replace(rdm1=c(atoms.rdm1), s1e=c(atoms.s1e))
    mo_occ0 = torch.as_tensor(atoms.mo_occ)
    nelecs = [int(round(float(mo_occ0[s, 0].sum()))) for s in range(2)]
    energy, fock = predict(params, atoms)
    atoms = atoms.replace(fock=fock, energy=energy)
    for _ in range(cycles):
        old_rdm1 = atoms.rdm1
        mo_energy, mo_coeff = solid_fock_solver(atoms.fock, atoms.s1e)
        mo_occ = solid_get_occ(mo_energy, nelecs)
        rdm1 = (1.0 - mixing_factor) * old_rdm1 + mixing_factor * solid_make_rdm1(mo_coeff, mo_occ)
        atoms = atoms.replace(mo_energy=mo_energy, mo_coeff=mo_coeff, mo_occ=mo_occ, rdm1=rdm1.resolve_conj())
        energy, fock = predict(params, atoms)
        atoms = atoms.replace(fock=fock, energy=energy)
    return atoms


def non_scf_predictor(functional, chunk_size: int = 1024, **kwargs) -> Callable:
    """evaluate.py:88-126: ``predictor(params, atoms) -> atoms`` with the energy and Fock matrix of
    ``energy_predictor`` at the given density (``chunk_size`` is accepted for signature compatibility)."""
    from .train import energy_predictor

    predict = energy_predictor(functional, **kwargs)

    def non_scf_predictor(params, atoms, *args):
        energy, fock = predict(params, atoms, *args)
        return atoms.replace(fock=fock, energy=energy)

    return non_scf_predictor


def simple_scf_loop(functional, mixing_factor: float = 0.4, chunk_size: int = 1024, cycles: int = 50,
                    start_cycle: int = 0, e_conv: float = 1e-5, g_conv: float = 1e-5, verbose: int = 0,
                    **kwargs) -> Callable:
    """evaluate.py:131-254: the non-jitted linear-mixing loop, as the reference runs it.

    Cycle 0 takes the incoming orbitals (no diagonalisation), occupies them and
    keeps their density matrix as the one to mix with, while the energy and
    Fock matrix are evaluated at the incoming rdm1; later cycles diagonalise the
    previous Fock matrix and mix.  Every cycle checks that the grid integral of
    the density matches atom_index.sum() - charge to 1e-3 (AssertionError
    otherwise).  All ``cycles`` run (``e_conv`` and ``g_conv`` are unused, as in
    the reference); ``chunk_size``, ``start_cycle`` and ``verbose`` are accepted
    for signature compatibility.
    """
    from .train import energy_predictor

    predict = energy_predictor(functional, **kwargs)

    def simple_scf_iterator(params, atoms, clip_cte=CLIP, *args):
        solid = getattr(atoms, "is_solid", False)
        dev = atoms.device
        nelectron = float(torch.as_tensor(atoms.atom_index).sum()) - float(atoms.charge)
        fock = atoms.fock
        old_rdm1 = None
        predicted_e = None
        for cycle in range(cycles):
            if cycle > 0:
                if solid:
                    mo_energy, mo_coeff = solid_fock_solver(fock, torch.as_tensor(atoms.s1e).to(dev, torch.complex128))
                else:
                    mo_energy, mo_coeff = safe_fock_solver(fock, engine.as_device_f64(atoms.s1e, dev))
                atoms = atoms.replace(mo_coeff=mo_coeff, mo_energy=mo_energy)
            atoms = atoms.replace(mo_occ=atoms.get_occ())
            if cycle == 0:
                old_rdm1 = atoms.make_rdm1()
            else:
                rdm1 = (1 - mixing_factor) * old_rdm1 + mixing_factor * atoms.make_rdm1()
                atoms = atoms.replace(rdm1=rdm1)
                old_rdm1 = rdm1
            w = engine.as_device_f64(atoms.grid.weights, dev)
            computed_charge = float(torch.einsum("r,rs->", w, atoms.density()))
            assert abs(nelectron - computed_charge) <= 1e-3 + 1e-5 * abs(computed_charge), (
                "Total charge is not conserved. given electrons: %.3f, computed electrons: %.3f"
                % (nelectron, computed_charge))
            predicted_e, fock = predict(params, atoms, *args)
        return atoms.replace(fock=fock, energy=predicted_e)

    return simple_scf_iterator


def diff_simple_scf_loop(functional, cycles: int = 25, mixing_factor: float = 0.4,
                         clip_cte: float = CLIP) -> Callable:
    """evaluate.py:256-344: returns ``iterator(params, atoms) -> atoms`` with the final
    rdm1, fock, energy, mo_coeff, mo_energy and mo_occ (a Molecule, or a Solid with
    k-points for constant-coefficient functionals)."""

    def iterator(params, atoms, *args):
        if getattr(atoms, "is_solid", False):
            return _solid_scf(functional, params, atoms, cycles, mixing_factor, clip_cte)
        atoms = _to_device(atoms)
        nelecs = [int(round(float(atoms.mo_occ[s].sum()))) for s in range(2)]
        energy, fock = energy_and_fock(functional, params, atoms, clip_cte)
        atoms = atoms.replace(fock=fock, energy=energy)
        for _ in range(cycles):
            old_rdm1 = atoms.rdm1
            mo_energy, mo_coeff = safe_fock_solver(atoms.fock, atoms.s1e)
            mo_occ = get_occ(mo_energy, nelecs)
            rdm1 = (1.0 - mixing_factor) * old_rdm1 + mixing_factor * make_rdm1(mo_coeff, mo_occ)
            atoms = atoms.replace(mo_energy=mo_energy, mo_coeff=mo_coeff, mo_occ=mo_occ, rdm1=rdm1)
            energy, fock = energy_and_fock(functional, params, atoms, clip_cte)
            atoms = atoms.replace(fock=fock, energy=energy)
        return atoms

    return iterator


class JittableDiis:
    """evaluate.py:1041-1210: CDIIS over a fixed history of ``max_diis`` entries, differentiable.

    F_DIIS = A^T (sum_i x_i F_i) A with x from the bordered system of the
    error inner products, e_i = A F_i D_i S A^T - (...)^T.  The history keeps
    the reference's indexing: entries are written at position ``cycle`` while
    cycle < max_diis, the one at cycle == max_diis is dropped (its scatter is
    out of bounds), and later ones shift the history by one.
    """

    def __init__(self, overlap_matrix, A, max_diis: int = 8):
        self.S, self.A, self.max_diis = overlap_matrix, A, int(max_diis)

    def empty(self, n_ao, like):
        z = lambda *shape: torch.zeros(shape, dtype=like.dtype, device=like.device)  # noqa: E731
        m = self.max_diis
        return z(m, 2, n_ao, n_ao), z(m, 2, n_ao, n_ao), z(m), z(m, 2, n_ao, n_ao)

    def _push(self, vec, x, cycle):
        if cycle > self.max_diis:
            return torch.cat((vec, x[None]), dim=0)[1:]
        if cycle < self.max_diis:
            return torch.cat((vec[:cycle], x[None], vec[cycle + 1:]), dim=0)
        return vec

    def update(self, new_data, diis_data, cycle):
        density, fock, energy = new_data
        dv, fv, ev, errv = diis_data
        fds = torch.einsum("ij,sjk,skl,lm,mn->sin", self.A, fock, density, self.S, self.A.T)
        err = fds - fds.transpose(1, 2)
        return (self._push(dv, density, cycle), self._push(fv, fock, cycle),
                self._push(ev, energy.reshape(()).to(ev.dtype), cycle), self._push(errv, err, cycle))

    def cdiis_minimize(self, error_vector, cycle):
        n = error_vector.shape[0]
        inner = torch.einsum("iskl,jskl->sij", error_vector, error_vector)
        used = (torch.arange(n, device=inner.device) <= cycle).to(inner.dtype)
        diag = torch.where(used > 0, torch.diagonal(inner, dim1=1, dim2=2), torch.ones_like(used))
        core = inner - torch.diag_embed(torch.diagonal(inner, dim1=1, dim2=2)) + torch.diag_embed(diag)
        border = used.expand(2, n)
        top = torch.cat((torch.zeros(2, 1, dtype=inner.dtype, device=inner.device), border), dim=1)
        B = torch.cat((top[:, None, :], torch.cat((border[:, :, None], core), dim=2)), dim=1)
        C = torch.zeros(n + 1, dtype=inner.dtype, device=inner.device)
        C[0] = 1.0
        x = torch.stack([_inv(B[s]) @ C for s in range(2)], dim=0)
        return x[:, 1:]

    def run(self, new_data, diis_data, cycle=0):
        diis_data = self.update(new_data, diis_data, cycle)
        _, fock_vector, _, error_vector = diis_data
        x = self.cdiis_minimize(error_vector, cycle)
        F = torch.einsum("si,isjk->sjk", x, fock_vector)
        return torch.einsum("ji,sjk,kl->sil", self.A, F, self.A), diis_data


def diff_scf_loop(functional, cycles: int = 25, clip_cte: float = CLIP, max_diis: int = 10) -> Callable:
    """evaluate.py:917-1038: ``iterator(params, atoms) -> atoms`` with CDIIS extrapolation of the
    Fock matrix (A = identity), the final rdm1, fock, energy, mo_coeff, mo_energy and mo_occ."""

    def iterator(params, atoms, *args):
        if getattr(atoms, "is_solid", False):
            # the reference's DIIS loops do not take k-points either: scf_loop rejects a Solid
            # (evaluate.py:402-403) and diff_scf_loop's A = identity(s1e.shape[0]) (evaluate.py:972)
            # does not fit k-point overlaps
            raise NotImplementedError("Solids with full BZ zampling not yet supported. Use simple_scf_loop or "
                                      "diff_simple_scf_loop instead.")
        atoms = _to_device(atoms)
        nelecs = [int(round(float(atoms.mo_occ[s].sum()))) for s in range(2)]
        energy, fock = energy_and_fock(functional, params, atoms, clip_cte)
        atoms = atoms.replace(fock=fock)
        n = fock.shape[-1]
        A = torch.eye(n, dtype=F64, device=fock.device)
        diis = JittableDiis(atoms.s1e, A, max_diis)
        diis_data = diis.empty(n, fock)
        for cycle in range(cycles):
            fock, diis_data = diis.run((atoms.rdm1, atoms.fock, energy), diis_data, cycle)
            mo_energy, mo_coeff = safe_fock_solver(fock, atoms.s1e)
            mo_occ = get_occ(mo_energy, nelecs)
            atoms = atoms.replace(fock=fock, mo_energy=mo_energy, mo_coeff=mo_coeff, mo_occ=mo_occ,
                                  rdm1=make_rdm1(mo_coeff, mo_occ))
            energy, fock = energy_and_fock(functional, params, atoms, clip_cte)
            atoms = atoms.replace(fock=fock)
        # The reference then runs one more iteration without DIIS history and
        # discards it (evaluate.py:1022-1031); the state it returns is this one.
        return atoms.replace(energy=energy)

    return iterator


# ------------------------------------------------------ orbital optimisers
def canonical_eigvec_signs(v: torch.Tensor) -> torch.Tensor:
    """Eigenvectors (columns) with their largest-magnitude component made positive."""
    idx = torch.argmax(v.abs(), dim=-2, keepdim=True)
    sign = torch.sign(torch.gather(v, -2, idx))
    return v * torch.where(sign == 0, torch.ones_like(sign), sign)


def _whitening(s1e, whitening: str):
    """evaluate.py:723-735: D with C = Q D for orthogonal Q (PCA, Cholesky or ZCA).

    PCA's D = diag(w^-1/2) v^T depends on the signs of the eigenvectors, which
    eigensolvers choose freely (the reference's result changes with its LAPACK);
    here each eigenvector is made to have its largest-magnitude component positive."""
    if whitening == "PCA":
        w, v = torch.linalg.eigh(s1e)
        return torch.diag(torch.sqrt(1.0 / w)) @ canonical_eigvec_signs(v).T
    if whitening == "Cholesky":
        return torch.linalg.cholesky(torch.linalg.inv(s1e)).T
    if whitening == "ZCA":
        w, v = torch.linalg.eigh(s1e)
        return v @ torch.diag(torch.sqrt(1.0 / w)) @ v.T
    raise ValueError(f"whitening must be 'PCA', 'Cholesky' or 'ZCA', got {whitening!r}")


def _orbital_energy(functional, params, atoms, W, D, clip_cte):
    """evaluate.py:640-692: E(W) with Q = qr(W_s), C = Q D, rdm1 = C occ C^T (differentiable in W)."""
    Q = torch.stack([torch.linalg.qr(W[0])[0], torch.linalg.qr(W[1])[0]])
    C = torch.einsum("sij,jk->ski", Q, D)
    rdm1 = make_rdm1(C, atoms.mo_occ)
    energy, _ = energy_and_fock(functional, params, atoms.replace(rdm1=rdm1, mo_coeff=C), clip_cte)
    return energy


def _orbital_setup(functional, params, atoms, clip_cte, whitening):
    if getattr(atoms, "is_solid", False):
        raise NotImplementedError("Solids with full BZ zampling not yet supported. Use simple_scf_loop instead.")
    atoms = _to_device(atoms)
    atoms = atoms.replace(mo_coeff=engine.as_device_f64(atoms.mo_coeff, atoms.device))
    with torch.no_grad():
        energy, _ = energy_and_fock(functional, params, atoms, clip_cte)
    D = _whitening(atoms.s1e, whitening)
    W = torch.einsum("sji,jk->sik", atoms.mo_coeff, torch.linalg.inv(D))  # C transposed
    return atoms, energy, D, W


def _orbital_step(functional, params, atoms, W, D, tx, opt_state, clip_cte):
    from .optim import apply_updates

    Wg = W.detach().requires_grad_(True)
    with torch.enable_grad():
        energy = _orbital_energy(functional, params, atoms, Wg, D, clip_cte)
        (grads,) = torch.autograd.grad(energy, [Wg])
    updates, opt_state = tx.update(grads, opt_state, W)
    return energy.detach(), apply_updates(W, updates), opt_state


def mol_orb_optimizer(fxc, tx, chunk_size: int = 1024, cycles: int = 500, e_conv: float = 1e-7,
                      whitening: str = "PCA", precision=None, verbose: int = 0, clip_cte: float = CLIP,
                      **kwargs) -> Callable:
    """evaluate.py:595-780: minimise the predicted energy over the density matrix generated by
    orthogonal orbitals C = qr(W) D (D4FT, Li et al., ICLR 2023), with the optax-protocol
    optimiser ``tx`` (``graddft_gb300.optim.adam``), until |dE| in kcal/mol <= e_conv or ``cycles``.

    As in the reference, the returned molecule carries the last evaluated energy (that of W
    before its final update) and keeps its other fields."""
    HARTREE2KCALMOL = 627.50947

    def neural_iterator(params, molecule, *args):
        atoms, predicted_e, D, W = _orbital_setup(fxc, params, molecule, clip_cte, whitening)
        old_e = float("inf")
        opt_state = tx.init(W)
        cycle = 0
        while abs(float(predicted_e) - old_e) * HARTREE2KCALMOL > e_conv and cycle < cycles:
            old_e = float(predicted_e)
            predicted_e, W, opt_state = _orbital_step(fxc, params, atoms, W, D, tx, opt_state, clip_cte)
            cycle += 1
            if verbose > 1:
                print(f"cycle: {cycle}, predicted energy: {float(predicted_e):.7e}, "
                      f"energy difference: {abs(float(predicted_e) - old_e):.4e}")
        return molecule.replace(energy=predicted_e)

    return neural_iterator


def jitted_mol_orb_optimizer(functional, tx, cycles: int = 500, clip_cte: float = CLIP, **kwargs) -> Callable:
    """evaluate.py:783-915: the same with PCA whitening and exactly ``cycles`` steps."""

    def neural_iterator(params, molecule, *args):
        atoms, predicted_e, D, W = _orbital_setup(functional, params, molecule, clip_cte, "PCA")
        opt_state = tx.init(W)
        for _ in range(cycles):
            predicted_e, W, opt_state = _orbital_step(functional, params, atoms, W, D, tx, opt_state, clip_cte)
        return molecule.replace(energy=predicted_e)

    return neural_iterator


# ------------------------------------------------------------ scf_loop
def mo_grads(mo_coeff, mo_occ, fock):
    """molecule.py:344-381 (orbital_grad as computed): sum over spins of C_vir^T F C_occ, with the
    columns of C zeroed where the orbital is (un)occupied; (n, n)."""
    c_occ = torch.where((mo_occ > 0)[:, None, :], mo_coeff, torch.zeros((), dtype=mo_coeff.dtype, device=mo_coeff.device))
    c_vir = torch.where((mo_occ == 0)[:, None, :], mo_coeff, torch.zeros((), dtype=mo_coeff.dtype, device=mo_coeff.device))
    return torch.einsum("sab,sac,scd->bd", c_vir, fock, c_occ)


def damping(s, d, f, factor):
    """evaluate.py:1477-1503 (PySCF's damping): f - (f0 + f0^T) factor / (factor + 1), f0 = (1 - s d) f d s."""
    f0 = (torch.eye(s.shape[0], dtype=s.dtype, device=s.device) - s @ d) @ f @ d @ s
    return f - (f0 + f0.T) * (factor / (factor + 1.0))


def level_shift(s, d, f, factor):
    """evaluate.py:1506-1545 (PySCF's level shift of the virtual space): f + (s - s d s) factor."""
    return f + (s - s @ d @ s) * factor


class Diis:
    """evaluate.py:1212-1386, the CDIIS branch: a history growing to ``max_diis`` entries (the
    oldest dropped beyond), error e_i = A F_i D_i S A^T - (...)^T, coefficients from the bordered
    matrix [[0, 1], [1, <e_i|e_j>]] inverted through its eigendecomposition, F = A^T (sum x_i F_i) A."""

    def __init__(self, overlap_matrix, A, max_diis: int = 8, diis_method: str = "CDIIS"):
        if diis_method != "CDIIS":
            raise NotImplementedError("only CDIIS is built: the reference's EDIIS/ADIIS minimise with "
                                      "jax.scipy.optimize.minimize")
        self.S, self.A, self.max_diis = overlap_matrix, A, int(max_diis)

    def update(self, new_data, diis_data):
        density, fock, energy = new_data
        dv, fv, ev, errv = diis_data
        fds = torch.einsum("ij,sjk,skl,lm,mn->sin", self.A, fock, density, self.S, self.A.T)
        err = fds - fds.transpose(1, 2)
        dv, fv = torch.cat((dv, density[None]), 0), torch.cat((fv, fock[None]), 0)
        ev, errv = torch.cat((ev, energy.reshape(1).to(ev.dtype))), torch.cat((errv, err[None]), 0)
        if errv.shape[0] > self.max_diis:
            dv, fv, ev, errv = dv[1:], fv[1:], ev[1:], errv[1:]
        return dv, fv, ev, errv

    def cdiis_minimize(self, error_vector):
        n = error_vector.shape[0]
        inner = torch.einsum("iskl,jskl->sij", error_vector, error_vector)
        B = torch.zeros((2, n + 1, n + 1), dtype=inner.dtype, device=inner.device)
        B[:, 1:, 1:] = inner
        B[:, 0, 1:] = 1.0
        B[:, 1:, 0] = 1.0
        xs = []
        for s in range(2):
            w, v = torch.linalg.eigh(B[s])
            xs.append(v @ torch.diag(1.0 / w) @ v.T[:, 0])  # B^-1 (1, 0, ..., 0)
        x = torch.stack(xs)
        if bool(torch.isnan(x).any()):
            raise AssertionError("DIIS coefficients are NaN")
        return x[:, 1:]

    def run(self, new_data, diis_data, cycle=0):
        diis_data = self.update(new_data, diis_data)
        fv, errv = diis_data[1], diis_data[3]
        if errv.shape[0] == 1:
            return fv[0], diis_data
        x = self.cdiis_minimize(errv)
        F = torch.einsum("si,isjk->sjk", x, fv)
        return torch.einsum("ji,sjk,kl->sil", self.A, F, self.A), diis_data


def scf_loop(functional, level_shift_factor=(0.0, 0.0), damp_factor=(0.0, 0.0), chunk_size: int = 1024,
             cycles: int = 50, diis_start_cycle: int = 0, e_conv: float = 1e-5, g_conv: float = 1e-5,
             diis_method: str = "CDIIS", smearing=None, smearing_sigma: float = 0.0, verbose: int = 0,
             **kwargs) -> Callable:
    """evaluate.py:355-592: the non-jitted SCF loop with CDIIS, damping and level shifting, until
    |dE| in kcal/mol <= e_conv and |orbital gradient| <= g_conv or ``cycles``; on convergence one more
    diagonalisation without level shift.  Every cycle checks the grid charge (AssertionError).
    Not built: EDIIS/ADIIS (``jax.scipy.optimize.minimize`` in the reference), smearing (the reference's
    smearing branch cannot run: it applies Python's min to a (2, n) array and stores a flattened
    occupation vector), and chi regeneration for omegas (the reference reads an undefined ``mf``)."""
    from .train import energy_predictor

    if smearing:
        raise NotImplementedError("smearing is not built (the reference's smearing branch cannot run as written)")
    predict = energy_predictor(functional, **kwargs)
    HARTREE2KCALMOL = 627.50947

    def _diag_occ_rdm1(molecule, fock, nelecs):
        mo_energy, mo_coeff = safe_fock_solver(fock, molecule.s1e)
        mo_occ = get_occ(mo_energy, nelecs)
        return molecule.replace(mo_coeff=mo_coeff, mo_energy=mo_energy, mo_occ=mo_occ,
                                rdm1=make_rdm1(mo_coeff, mo_occ))

    def scf_iterator(params, molecule, *args):
        if getattr(molecule, "is_solid", False):
            raise NotImplementedError("Solids with full BZ zampling not yet supported. Use simple_scf_loop or "
                                      "diff_simple_scf_loop instead.")
        if getattr(molecule, "omegas", None):
            raise NotImplementedError("chi regeneration inside scf_loop is not built")
        molecule = _to_device(molecule)
        dev = molecule.device
        nelectron = float(torch.as_tensor(molecule.atom_index).sum()) - float(molecule.charge)
        nelecs = [int(round(float(molecule.mo_occ[s].sum()))) for s in range(2)]
        old_e, norm_gorb, cycle = float("inf"), float("inf"), 0
        predicted_e, fock = predict(params, molecule, *args)
        n = molecule.s1e.shape[0]
        A = torch.eye(n, dtype=F64, device=dev)
        diis = Diis(molecule.s1e, A, max_diis=10, diis_method=diis_method)
        z = torch.zeros((0, 2, n, n), dtype=F64, device=dev)
        diis_data = (z, z, torch.zeros(0, dtype=F64, device=dev), z)
        while ((abs(float(predicted_e) - old_e) * HARTREE2KCALMOL > e_conv or norm_gorb > g_conv)
               and cycle < cycles):
            old_e = float(predicted_e)
            if 0 <= cycle < diis_start_cycle - 1 and abs(damp_factor[0]) + abs(damp_factor[1]) > 1e-4:
                fock = torch.stack([damping(molecule.s1e, molecule.rdm1[s], fock[s], damp_factor[s]) for s in range(2)])
            if cycle >= diis_start_cycle:
                fock, diis_data = diis.run((molecule.rdm1, fock, predicted_e), diis_data, cycle)
            if abs(level_shift_factor[0]) + abs(level_shift_factor[1]) > 1e-4:
                fock = torch.stack([level_shift(molecule.s1e, molecule.rdm1[s], fock[s], level_shift_factor[s])
                                    for s in range(2)])
            molecule = _diag_occ_rdm1(molecule, fock, nelecs)
            w = engine.as_device_f64(molecule.grid.weights, dev)
            computed_charge = float(torch.einsum("r,rs->", w, molecule.density()))
            assert abs(nelectron - computed_charge) <= 1e-3 + 1e-5 * abs(computed_charge), \
                "Total charge is not conserved"
            predicted_e, fock = predict(params, molecule, *args)
            norm_gorb = float(torch.linalg.norm(mo_grads(molecule.mo_coeff, molecule.mo_occ, fock)))
            if verbose > 1:
                print(f"cycle: {cycle}, energy: {float(predicted_e):.7e}, "
                      f"energy difference: {abs(float(predicted_e) - old_e):.4e}, norm_gradient_orbitals: {norm_gorb:.2e}")
            cycle += 1
        if abs(float(predicted_e) - old_e) * HARTREE2KCALMOL < e_conv and norm_gorb < g_conv:
            molecule = _diag_occ_rdm1(molecule, fock, nelecs)  # once more, without the level shift
            predicted_e, fock = predict(params, molecule, *args)
        return molecule.replace(fock=fock, energy=predicted_e)

    return scf_iterator
