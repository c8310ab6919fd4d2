"""Solid (k-point) containers and their XC path (solid.py:34-674 of the reference).

A ``Solid`` holds complex crystal AOs per k-point, ``ao`` (n_kpt, grid, n),
``grad_ao`` (n_kpt, grid, n, 3), ``grad_n_ao[2]`` (n_kpt, grid, n, 3), and a
complex density matrix ``rdm1`` (2, n_kpt, n, n).  The reference's densities are
unconjugated bilinear forms summed over k-points with the weights of
``KPointInfo`` (solid.py:491-632), e.g.

    rho_s(r) = Re sum_k w_k sum_ab D_s,k[a, b] phi_k,a(r) phi_k,b(r).

Each k-point is packed once as a real molecule of 2n functions
[Re phi_k | Im phi_k]; the library evaluates the forms on the doubled basis
with the real matrix w_k [[Re D, -Im D], [-Im D, -Re D]], sums the features over
k-points, runs the point kernel once, and returns jax.grad's complex gradient
of E_xc (dE/dRe D - i dE/dIm D) per k-point.  Both arithmetic forms apply.
"""
from __future__ import annotations

import ctypes
import dataclasses
from dataclasses import dataclass, field
from typing import Any, List, Optional

import torch

from . import _lib, engine
from .molecule import Grid

C128 = torch.complex128
F64 = torch.float64

_AO_FIELDS = ("grid", "kpt_info", "ao", "grad_ao", "grad_n_ao", "precision")


@dataclass
class KPointInfo:
    """solid.py:71-98."""

    kpts_abs: Any
    kpts_scaled: Any
    weights: Any

    def to_dict(self) -> dict:
        return {"kpts_abs": self.kpts_abs, "kpts_scaled": self.kpts_scaled, "kpt_weights": self.weights}


def _as_c128(x, dev) -> torch.Tensor:
    if x is None:
        return None
    if not isinstance(x, torch.Tensor):
        x = torch.as_tensor(x)
    return x.to(device=dev, dtype=C128).resolve_conj().contiguous()


def _real_tables(x: torch.Tensor) -> torch.Tensor:
    """(grid, n[, 3]) complex -> (grid, 2n[, 3]) real: [Re | Im] along the orbital axis."""
    return torch.cat((x.real, x.imag), dim=1).contiguous()


class KPointResident:
    """The k-points of a Solid resident in HBM: one library molecule of 2n functions per k-point."""

    def __init__(self, ao, grad_ao, grad2_ao, weights, kweights, precision="fp64", device=None):
        dev = engine.require_cuda(device)
        self.device = dev
        ao = _as_c128(ao, dev)
        grad_ao = _as_c128(grad_ao, dev)
        grad2_ao = _as_c128(grad2_ao, dev)
        n_kpt, n_grid, n = ao.shape
        if grad_ao.shape != (n_kpt, n_grid, n, 3):
            raise ValueError(f"grad_ao {tuple(grad_ao.shape)} does not match ({n_kpt}, {n_grid}, {n}, 3)")
        if grad2_ao is not None and grad2_ao.shape != (n_kpt, n_grid, n, 3):
            raise ValueError(f"grad_n_ao[2] {tuple(grad2_ao.shape)} does not match ({n_kpt}, {n_grid}, {n}, 3)")
        self.n_kpt, self.n_grid, self.n = n_kpt, n_grid, n
        self.kweights = [float(w) for w in torch.as_tensor(kweights).reshape(-1).tolist()]
        if len(self.kweights) != n_kpt:
            raise ValueError(f"{len(self.kweights)} k-point weights for {n_kpt} k-points")
        self.kw_host = (ctypes.c_double * n_kpt)(*self.kweights)
        self.kw_dev = torch.tensor(self.kweights, dtype=F64, device=dev)
        self.mols = [engine.Resident.from_tables(_real_tables(ao[k]), _real_tables(grad_ao[k]),
                                                 None if grad2_ao is None else _real_tables(grad2_ao[k]), weights,
                                                 precision, dev) for k in range(n_kpt)]
        self.descs = (_lib.GdftMolecule * n_kpt)(*[m.desc for m in self.mols])
        nbytes = ctypes.c_size_t()
        _lib.check(_lib.load().gdft_kpoint_workspace_bytes(self.descs, n_kpt, ctypes.byref(nbytes)))
        self.ws = torch.zeros(nbytes.value, dtype=torch.uint8, device=dev)

    def _rdm1(self, rdm1) -> torch.Tensor:
        d = _as_c128(rdm1, self.device)
        if d.shape != (2, self.n_kpt, self.n, self.n):
            raise ValueError(f"rdm1 must be (2, {self.n_kpt}, {self.n}, {self.n}), got {tuple(d.shape)}")
        return d

    def density(self, rdm1, want=("rho", "grad_rho", "lapl", "tau")):
        d = self._rdm1(rdm1)
        n = self.n_grid
        out = {
            "rho": torch.empty((n, 2), dtype=F64, device=self.device) if "rho" in want else None,
            "grad_rho": torch.empty((n, 2, 3), dtype=F64, device=self.device) if "grad_rho" in want else None,
            "lapl": torch.empty((n, 2), dtype=F64, device=self.device) if "lapl" in want else None,
            "tau": torch.empty((n, 2), dtype=F64, device=self.device) if "tau" in want else None,
        }
        P = engine._ptr
        _lib.check(_lib.load().gdft_kpoint_density(self.descs, self.n_kpt, P(torch.view_as_real(d)), self.kw_host,
                                                   P(out["rho"]), P(out["grad_rho"]), P(out["lapl"]), P(out["tau"]),
                                                   P(self.ws), self.ws.numel(), engine._stream(self.device)))
        return out

    def xc_energy_and_grads(self, rdm1, fn, ehf=None, want_vxc=True):
        if ehf is not None:
            raise NotImplementedError("Hartree-Fock methods (for computation of Hybrid functionals) will come in a "
                                      "later release.")
        d = self._rdm1(rdm1)
        exc = torch.empty((), dtype=F64, device=self.device)
        vxc = torch.empty_like(d) if want_vxc else None
        P = engine._ptr
        _lib.check(_lib.load().gdft_kpoint_xc_energy_and_grads(
            self.descs, self.n_kpt, P(torch.view_as_real(d)), self.kw_host, ctypes.byref(fn), P(exc),
            None if vxc is None else P(torch.view_as_real(vxc)), P(self.ws), self.ws.numel(),
            engine._stream(self.device)))
        return exc, vxc

    def coulomb(self, rep_tensor, rdm1, h1e=None, nuclear_repulsion=0.0, want_energy=False):
        d = self._rdm1(rdm1)
        rep = _as_c128(rep_tensor, self.device)
        K, n = self.n_kpt, self.n
        if rep is None or rep.shape != (K, K, n, n, n, n):
            raise ValueError(f"rep_tensor must be ({K}, {K}, {n}, {n}, {n}, {n})")
        h = _as_c128(h1e, self.device)
        if want_energy and (h is None or h.shape != (K, n, n)):
            raise ValueError(f"h1e must be ({K}, {n}, {n})")
        vj = torch.empty((K, n, n), dtype=C128, device=self.device)
        e = torch.empty((), dtype=F64, device=self.device) if want_energy else None
        P = engine._ptr
        _lib.check(_lib.load().gdft_kpoint_coulomb(K, n, P(torch.view_as_real(rep)), P(torch.view_as_real(d)),
                                                   None if not want_energy else P(torch.view_as_real(h)),
                                                   P(self.kw_dev), float(nuclear_repulsion),
                                                   P(torch.view_as_real(vj)), P(e), engine._stream(self.device)))
        return vj, e

    def fock(self, h1e, vj, vxc, clip):
        h = _as_c128(h1e, self.device)
        out = torch.empty_like(vxc)
        P = engine._ptr
        _lib.check(_lib.load().gdft_kpoint_fock(self.n_kpt, self.n, P(torch.view_as_real(h)),
                                                P(torch.view_as_real(vj.contiguous())),
                                                P(torch.view_as_real(vxc.contiguous())), float(clip),
                                                P(torch.view_as_real(out)), engine._stream(self.device)))
        return out


@dataclass
class Solid:
    """solid.py:100-270 (the fields the XC path and predict read)."""

    grid: Grid
    kpt_info: KPointInfo
    atom_index: Any
    lattice_vectors: Any
    nuclear_pos: Any
    ao: Any
    grad_ao: Any
    grad_n_ao: Any
    rdm1: Any
    nuclear_repulsion: Any
    h1e: Any
    vj: Any
    mo_coeff: Any
    mo_occ: Any
    mo_energy: Any
    mf_energy: Optional[Any] = None
    s1e: Optional[Any] = None
    omegas: Optional[Any] = None
    chi: Optional[Any] = None
    rep_tensor: Optional[Any] = None
    energy: Optional[Any] = None
    basis: Optional[Any] = None
    name: Optional[Any] = None
    spin: Optional[Any] = 0
    charge: Optional[Any] = 0
    unit_Angstrom: Optional[bool] = True
    grid_level: Optional[Any] = 2
    scf_iteration: Optional[Any] = 50
    fock: Optional[Any] = None
    precision: str = "fp64"
    _resident: Any = field(default=None, compare=False, repr=False)

    is_solid = True

    @property
    def device(self) -> torch.device:
        t = self.ao if isinstance(self.ao, torch.Tensor) else None
        return engine.require_cuda(t.device if t is not None and t.is_cuda else None)

    def resident(self) -> KPointResident:
        if self._resident is None:
            g2 = None
            if self.grad_n_ao is not None:
                g2 = self.grad_n_ao[2] if isinstance(self.grad_n_ao, (dict, list, tuple)) else self.grad_n_ao
            r = KPointResident(self.ao, self.grad_ao, g2, self.grid.weights, self.kpt_info.weights, self.precision,
                               self.device)
            object.__setattr__(self, "_resident", r)
        return self._resident

    def replace(self, **kwargs) -> "Solid":
        keep = self._resident if not any(k in kwargs for k in _AO_FIELDS) else None
        kwargs.setdefault("_resident", keep)
        return dataclasses.replace(self, **kwargs)

    def _rdm1(self):
        return _as_c128(self.rdm1, self.device)

    def to_dict(self) -> dict:
        rest = {f.name: getattr(self, f.name) for f in dataclasses.fields(self)[2:] if f.name != "_resident"}
        return dict(**self.grid.to_dict(), **self.kpt_info.to_dict(), **rest)

    # ------------------------------------------------- density primitives
    def density(self, *args, **kwargs):
        """solid.py:140-147 / 491-521 -> (grid, spin)."""
        return self.resident().density(self._rdm1(), want=("rho",))["rho"]

    def grad_density(self, *args, **kwargs):
        """solid.py:179-186 / 523-558 -> (grid, spin, 3)."""
        return self.resident().density(self._rdm1(), want=("grad_rho",))["grad_rho"]

    def lapl_density(self, *args, **kwargs):
        """solid.py:188-195 / 560-598 -> (grid, spin)."""
        return self.resident().density(self._rdm1(), want=("lapl",))["lapl"]

    def kinetic_density(self, *args, **kwargs):
        """solid.py:197-204 / 600-632 -> (grid, spin)."""
        return self.resident().density(self._rdm1(), want=("tau",))["tau"]

    # --------------------------------------------------------- non-XC parts
    def get_coulomb_potential(self, *args, **kwargs):
        """solid.py:218-226 / 302-330: (n_kpt, n, n) complex."""
        vj, _ = self.resident().coulomb(self.rep_tensor, self._rdm1())
        return vj

    def nonXC(self, *args, **kwargs):
        """solid.py:149-156 / 367-411."""
        _, e = self.resident().coulomb(self.rep_tensor, self._rdm1(), self.h1e, float(self.nuclear_repulsion),
                                       want_energy=True)
        return e

    # ------------------------------------------------------------- SCF
    def make_rdm1(self, *args, **kwargs):
        """solid.py:158-165 / 413-435."""
        from .scf import solid_make_rdm1

        return solid_make_rdm1(_as_c128(self.mo_coeff, self.device), torch.as_tensor(self.mo_occ).to(self.device))

    def get_occ(self):
        """solid.py:167-177 / 438-487 (electrons per spin from the first k-point of mo_occ)."""
        from .scf import solid_get_occ

        mo_occ = torch.as_tensor(self.mo_occ)
        nelecs = [int(round(float(mo_occ[s, 0].sum()))) for s in range(2)]
        return solid_get_occ(torch.as_tensor(self.mo_energy).to(self.device), nelecs)

    # ------------------------------------------------- exact exchange
    def select_HF_omegas(self, omegas):
        raise NotImplementedError("Hartree-Fock methods (for computation of Hybrid functionals) will come in a "
                                  "later release.")

    def HF_energy_density(self, omegas, *args, **kwargs):
        raise NotImplementedError("Hartree-Fock methods (for computation of Hybrid functionals) will come in a "
                                  "later release.")

    def HF_density_grad_2_Fock(self, *args, **kwargs):
        raise NotImplementedError("Hartree-Fock methods (for computation of Hybrid functionals) will come in a "
                                  "later release.")

    def HF_coefficient_input_grad_2_Fock(self, *args, **kwargs):
        raise NotImplementedError("Hartree-Fock methods (for computation of Hybrid functionals) will come in a "
                                  "later release.")
