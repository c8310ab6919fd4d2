"""Grid and Molecule containers with the reference's field names (molecule.py:34-336).

A ``Molecule`` keeps its arrays as CUDA tensors and lazily packs its grid and
AO tables once into the library's resident layout; ``replace`` shares that
resident copy while the grid and AO fields are unchanged (as in an SCF loop or
a training step, where only ``rdm1`` and the parameters change).
"""
from __future__ import annotations

import dataclasses
from dataclasses import dataclass, field
from typing import Any, Optional

import torch

from . import engine

_AO_FIELDS = ("grid", "ao", "grad_ao", "grad_n_ao", "precision")
# clip_cte of the HF Fock-term gradients when the caller passes none (molecule.py:206-294 default).
HF_GRAD_CLIP = 1e-30


@dataclass(frozen=True)
class Grid:
    """molecule.py:34-69."""

    coords: Any
    weights: Any

    def __len__(self):
        return int(self.weights.shape[0])

    def to_dict(self) -> dict:
        return {"coords": self.coords, "weights": self.weights}

    def integrate(self, vals, axis: int = 0):
        """molecule.py:45-69: tensordot(weights, vals, axes=(0, axis))."""
        return torch.tensordot(self.weights, vals, dims=([0], [axis]))


@dataclass(frozen=True)
class Molecule:
    """molecule.py:72-336 (the fields the XC path and predict read)."""

    grid: Grid
    atom_index: Any
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
    # Extensions: stop-gradient HF energy densities (omega, spin, grid) supplied
    # directly when no chi tensor is available, and the arithmetic form.
    ehf: Optional[Any] = None
    # Three-index density-fitting Coulomb tensor (naux, ao, ao), used for J
    # when a four-index rep_tensor is too large to hold.
    df_tensor: Optional[Any] = None
    precision: str = "fp64"
    _resident: Any = field(default=None, compare=False, repr=False)

    # ------------------------------------------------------------ plumbing
    @property
    def grid_size(self):
        return len(self.grid)

    @property
    def device(self) -> torch.device:
        t = self.ao if isinstance(self.ao, torch.Tensor) else None
        return engine.require_cuda(t.device if t is not None and t.is_cuda else None)

    def resident(self) -> engine.Resident:
        if self._resident is None:
            g2 = None
            if self.grad_n_ao is not None:
                g2 = self.grad_n_ao[2] if isinstance(self.grad_n_ao, (dict, list, tuple)) else self.grad_n_ao
            r = engine.Resident.from_tables(self.ao, self.grad_ao, g2, self.grid.weights, self.precision,
                                            self.device)
            object.__setattr__(self, "_resident", r)
        return self._resident

    def replace(self, **kwargs) -> "Molecule":
        keep = self._resident if not any(k in kwargs for k in _AO_FIELDS) else None
        kwargs.setdefault("_resident", keep)
        return dataclasses.replace(self, **kwargs)

    def _rdm1(self):
        return engine.as_device_f64(self.rdm1, self.device)

    # ------------------------------------------------- density primitives
    def density(self, *args, **kwargs):
        """molecule.py:117-124 -> (grid, spin)."""
        return self.resident().density(self._rdm1(), want=("rho",))["rho"]

    def grad_density(self, *args, **kwargs):
        """molecule.py:126-133 -> (grid, spin, 3)."""
        return self.resident().density(self._rdm1(), want=("grad_rho",))["grad_rho"]

    def lapl_density(self, *args, **kwargs):
        """molecule.py:135-142 -> (grid, spin)."""
        return self.resident().density(self._rdm1(), want=("lapl",))["lapl"]

    def kinetic_density(self, *args, **kwargs):
        """molecule.py:144-151 -> (grid, spin)."""
        return self.resident().density(self._rdm1(), want=("tau",))["tau"]

    # ------------------------------------------------------------- orbitals
    def make_rdm1(self, *args, **kwargs):
        """molecule.py:816-846: D_s = C_s diag(occ_s) C_s^T."""
        from .scf import make_rdm1

        dev = self.device
        return make_rdm1(engine.as_device_f64(self.mo_coeff, dev), engine.as_device_f64(self.mo_occ, dev))

    def get_occ(self):
        """molecule.py:848-889: the nelec lowest orbitals of each spin, nelec from mo_occ."""
        from .scf import get_occ

        mo_occ = torch.as_tensor(self.mo_occ)
        nelecs = [int(round(float(mo_occ[s].sum()))) for s in range(2)]
        return get_occ(engine.as_device_f64(self.mo_energy, self.device), nelecs)

    def get_mo_grads(self, *args, **kwargs):
        """molecule.py:258-266 / 344-381: the orbital gradient as the reference computes it."""
        from .scf import mo_grads

        dev = self.device
        return mo_grads(engine.as_device_f64(self.mo_coeff, dev), engine.as_device_f64(self.mo_occ, dev),
                        engine.as_device_f64(self.fock, dev))

    # --------------------------------------------------------- non-XC parts
    def get_coulomb_potential(self, *args, **kwargs):
        """molecule.py:110-115: J from rep_tensor and rdm1 summed over spin."""
        vj, _ = engine.coulomb(self.rep_tensor, self._rdm1())
        return vj

    def nonXC(self, *args, **kwargs):
        """molecule.py:296-298."""
        _, e = engine.coulomb(self.rep_tensor, self._rdm1(), self.h1e, float(self.nuclear_repulsion),
                              want_energy=True)
        return e

    # ------------------------------------------------- exact exchange (chi)
    def select_HF_omegas(self, omegas):
        """molecule.py:153-183: chi (grid, omega, spin, orbitals) for the given omegas."""
        if self.chi is None:
            raise ValueError("Precomputed chi tensor has not been loaded.")
        have = [float(o) for o in (self.omegas.tolist() if hasattr(self.omegas, "tolist") else self.omegas)]
        for o in omegas:
            if float(o) not in have:
                raise ValueError(f"The molecule.chi tensor does not contain omega value {o}, only {self.omegas}")
        idx = [have.index(float(o)) for o in omegas]
        chi = engine.as_device_f64(self.chi, self.device)
        if idx == list(range(chi.shape[1])) and chi.is_contiguous():
            return chi  # every omega in stored order: no gather (callers only read chi)
        return chi[:, idx].contiguous()

    def HF_energy_density(self, omegas, *args, **kwargs):
        """molecule.py:185-204: ehf (omega, spin, grid) from chi on the device.

        Without chi, a supplied stop-gradient ``ehf`` (omega, spin, grid) stands in.
        """
        if self.chi is not None:
            return engine.hf_energy_density(engine.as_device_f64(self.ao, self.device), self._rdm1(),
                                            self.select_HF_omegas(omegas), form=self.precision)
        if self.ehf is not None:
            return engine.as_device_f64(self.ehf, self.device)[: len(omegas)]
        raise ValueError("Precomputed chi tensor has not been loaded.")

    def HF_density_grad_2_Fock(self, functional, params, omegas, ehf, coefficient_inputs, densities_wout_hf,
                               **kwargs):
        """molecule.py:206-250 -> (omega, spin, orbitals, orbitals).

        F[w,s,a,b] = -1/2 sum_r chi[r,w,s,b] g[w,s,r] ao[r,a] with g = dE_xc/d ehf
        through the densities (molecule.py:545-613).  The densities are
        recomputed on the device from rdm1 (they are the ones predict passes).
        """
        chi = self.select_HF_omegas(omegas)
        g = functional.hf_density_gradient(params, self, engine.as_device_f64(ehf, self.device),
                                           kwargs.get("clip_cte", HF_GRAD_CLIP))
        return self._hf_fock_per_omega(chi, g)

    def _hf_fock_per_omega(self, chi, g):
        ao = engine.as_device_f64(self.ao, self.device)
        return torch.stack([engine.hf_fock(ao, chi[:, w:w + 1], g[w:w + 1], form=self.precision)
                            for w in range(chi.shape[1])])

    def _hf_fock_omega_sum(self, chi, g):
        """The omega sum of ``_hf_fock_per_omega`` as one contraction (B = -1/2 sum_w g chi before the GEMM),
        on the stored chi without per-omega copies."""
        return engine.hf_fock(engine.as_device_f64(self.ao, self.device), chi, g, form=self.precision)

    def HF_coefficient_input_grad_2_Fock(self, functional, params, omegas, ehf, cinputs_wout_hf, densities,
                                         **kwargs):
        """molecule.py:252-294 -> (omega, spin, orbitals, orbitals): as HF_density_grad_2_Fock with
        g = dE_xc/d ehf through the network's HF inputs (molecule.py:668-673)."""
        chi = self.select_HF_omegas(omegas)
        g = functional.hf_cinput_gradient(params, self, engine.as_device_f64(ehf, self.device),
                                          kwargs.get("clip_cte", HF_GRAD_CLIP))
        return self._hf_fock_per_omega(chi, g)

    def to_dict(self) -> dict:
        d = {f.name: getattr(self, f.name) for f in dataclasses.fields(self)[1:] if not f.name.startswith("_")}
        return dict(**self.grid.to_dict(), **d)


def _resident_for(rdm1, ao, grad_ao=None, grad2_ao=None):
    dev = engine.require_cuda(ao.device if isinstance(ao, torch.Tensor) and ao.is_cuda else None)
    ao = engine.as_device_f64(ao, dev)
    n, m = ao.shape
    g = engine.as_device_f64(grad_ao, dev) if grad_ao is not None else torch.zeros((n, m, 3), dtype=torch.float64,
                                                                                     device=dev)
    w = torch.ones(n, dtype=torch.float64, device=dev)
    return engine.Resident.from_tables(ao, g, grad2_ao, w, "fp64", dev)


def density(rdm1, ao, *args, **kwargs):
    """molecule.py:385-409 (free function)."""
    return _resident_for(rdm1, ao).density(rdm1, want=("rho",))["rho"]


def grad_density(rdm1, ao, grad_ao, *args, **kwargs):
    """molecule.py:411-440 (free function)."""
    return _resident_for(rdm1, ao, grad_ao).density(rdm1, want=("grad_rho",))["grad_rho"]


def lapl_density(rdm1, ao, grad_ao, grad_2_ao, *args, **kwargs):
    """molecule.py:442-474 (free function)."""
    return _resident_for(rdm1, ao, grad_ao, grad_2_ao).density(rdm1, want=("lapl",))["lapl"]


def kinetic_density(rdm1, grad_ao, *args, **kwargs):
    """molecule.py:476-502 (free function)."""
    ao = torch.zeros(grad_ao.shape[:2], dtype=torch.float64, device=grad_ao.device)
    return _resident_for(rdm1, ao, grad_ao).density(rdm1, want=("tau",))["tau"]


def abs_clip(arr, threshold):
    """molecule.py:687-689."""
    return torch.where(arr.abs() > threshold, arr, torch.zeros((), dtype=arr.dtype, device=arr.device))
