"""Functional plugin API with the reference's slots (functional.py:48-342).

A ``Functional`` is described exactly as in the reference (``coefficients``,
``energy_densities``, ``nograd_densities``, ``combine_densities`` ...).  The
energy-density callables this package provides (``lsda_density``,
``b88_density`` ... and ``stack_densities`` of them) are recognised and mapped
to columns of the fused device kernels; an unknown callable raises
``NotImplementedError`` - there is no eager or CPU fallback.
"""
from __future__ import annotations

import functools
from dataclasses import dataclass
from typing import Any, Callable, Optional, Sequence

import numpy as np
import torch

from . import _lib, engine

CLIP = 1e-30


def energy_density_columns(fn) -> tuple:
    """The device columns of a known energy-density callable.

    ``functools.partial(dm21_densities, functional_type=...)`` and the same of
    ``densities`` (how the reference's examples select the feature set, e.g.
    examples/article_experiments/train_atoms.py:93) resolve through the bound
    keywords."""
    if isinstance(fn, functools.partial) and getattr(fn.func, "_gdft_cols_of", None) is not None:
        if fn.args:
            raise NotImplementedError(f"{fn.func.__name__}: bind functional_type / clip_cte as keywords")
        kw = dict(fn.keywords)
        if float(kw.pop("clip_cte", CLIP)) != CLIP:
            raise NotImplementedError(f"{fn.func.__name__}: energy densities evaluate with clip_cte={CLIP}")
        return tuple(fn.func._gdft_cols_of(**kw))
    cols = getattr(fn, "_gdft_cols", None)
    if cols is None:
        raise NotImplementedError(
            f"energy-density callable {getattr(fn, '__name__', fn)!r} has no device kernel; use the ones in "
            "graddft_gb300.popular_functionals / graddft_gb300.functional or stack_densities() of them")
    return tuple(cols)


def tag_columns(*cols):
    def deco(f):
        f._gdft_cols = tuple(cols)
        return f

    return deco


def stack_densities(*fns) -> Callable:
    """A callable stacking the columns of several known energy-density callables (jnp.concatenate axis=1)."""
    cols = sum((energy_density_columns(f) for f in fns), ())

    @tag_columns(*cols)
    def stacked(molecule, clip_cte: float = CLIP, *_, **__):
        return molecule_energy_densities(molecule, cols, clip_cte)

    stacked.__name__ = "stack_densities(" + ", ".join(getattr(f, "__name__", "?") for f in fns) + ")"
    return stacked


def molecule_energy_densities(molecule, cols: Sequence[int], clip_cte: float = CLIP, ehf=None):
    """Raw energy-density columns (grid, F) of a molecule, computed on the device."""
    r = molecule.resident()
    fn = engine.make_functional(cols, [1.0], clip_cte)
    ehf_t = engine.as_device_f64(ehf if ehf is not None else getattr(molecule, "ehf", None), r.device)
    needs_hf = any(c in (_lib.COL_HF, _lib.COL_HF_W0, _lib.COL_HF_W1) for c in cols)
    if not needs_hf:
        ehf_t = None
    out = torch.empty((r.n_grid, len(cols)), dtype=torch.float64, device=r.device)
    import ctypes
    n_omega = 0 if ehf_t is None else ehf_t.shape[0]
    _lib.check(_lib.load().gdft_energy_densities(ctypes.byref(r.desc), engine._ptr(molecule._rdm1()),
                                                 ctypes.byref(fn), engine._ptr(ehf_t), n_omega, engine._ptr(out),
                                                 engine._ptr(r.ws), r.ws.numel(), engine._stream(r.device)))
    return out


def _const_row(c) -> list:
    a = np.asarray(c.detach().cpu().numpy() if isinstance(c, torch.Tensor) else c, dtype=np.float64)
    if a.ndim == 2 and a.shape[0] == 1:
        a = a[0]
    if a.ndim != 1:
        raise NotImplementedError("only constant coefficient rows are supported for non-neural functionals")
    return [float(x) for x in a]


class _XcEnergy(torch.autograd.Function):
    """E_xc(D) with dE_xc/dD from the fused device path (train.py:86 value_and_grad)."""

    @staticmethod
    def forward(ctx, rdm1, resident, fn, ehf):
        exc, vxc = resident.xc_energy_and_grads(rdm1.detach(), fn, ehf, want_vxc=True)
        ctx.save_for_backward(vxc)
        return exc

    @staticmethod
    def backward(ctx, g):
        (vxc,) = ctx.saved_tensors
        return g * vxc, None, None, None


class _XcEnergyPotential(torch.autograd.Function):
    """(E_xc, V_xc) from one device pass; E_xc is differentiable in rdm1 (its gradient is V_xc).  A
    gradient flowing into V_xc would need the functional's second derivative, which is built for the
    DM21 network (NeuralFunctional) only."""

    @staticmethod
    def forward(ctx, rdm1, resident, fn, ehf):
        exc, vxc = resident.xc_energy_and_grads(rdm1.detach(), fn, ehf, want_vxc=True)
        ctx.save_for_backward(vxc)
        return exc, vxc

    @staticmethod
    def backward(ctx, g_exc, g_vxc):
        (vxc,) = ctx.saved_tensors
        if g_vxc is not None and bool(torch.any(g_vxc != 0)):
            raise NotImplementedError("second derivatives of constant-coefficient functionals are not built; "
                                      "differentiate through V_xc with a NeuralFunctional (DM21)")
        return (None if g_exc is None else g_exc * vxc), None, None, None


@dataclass
class Functional:
    """functional.py:48-342."""

    coefficients: Callable
    energy_densities: Optional[Callable] = None
    coefficient_inputs: Optional[Callable] = None
    nograd_densities: Optional[Callable] = None
    densitygrads: Optional[Callable] = None
    combine_densities: Optional[Callable] = None
    nograd_coefficient_inputs: Optional[Callable] = None
    coefficient_input_grads: Optional[Callable] = None
    combine_inputs: Optional[Callable] = None
    is_xc: bool = True
    exchange_mask: Any = None

    # -------------------------------------------------------------- flax-like
    def __call__(self, coefficient_inputs):
        return self.coefficients(self, coefficient_inputs)

    def apply(self, params, coefficient_inputs, **kwargs):
        return self.coefficients(self, coefficient_inputs)

    # ----------------------------------------------------------- dispatching
    def _columns(self, atoms):
        """Columns and the stop-gradient HF input of compute_densities (functional.py:160-185)."""
        cols: tuple = ()
        ehf = None
        if self.energy_densities is not None:
            cols = energy_density_columns(self.energy_densities)
        if self.nograd_densities is not None:
            ehf = self.nograd_densities(atoms)
            comb = self.combine_densities
            hf_cols = getattr(comb, "_gdft_hf_cols", None) if comb is not None else None
            if hf_cols is None:
                raise NotImplementedError("combine_densities must be one of the known combine functions")
            cols = cols + tuple(hf_cols)
        if not cols:
            raise ValueError("functional has no energy densities")
        return cols, ehf

    def spec(self, params, atoms, clip_cte: float = CLIP):
        cols, ehf = self._columns(atoms)
        if self.coefficient_inputs is not None or self.nograd_coefficient_inputs is not None:
            raise NotImplementedError("coefficient inputs are only supported by NeuralFunctional/DM21")
        coeffs = _const_row(self.coefficients(self, None))
        return engine.make_functional(cols, coeffs, clip_cte), ehf

    # --------------------------------------------------------------- the API
    def compute_densities(self, atoms, clip_cte: float = CLIP, *args, **kwargs):
        cols, ehf = self._columns(atoms)
        dens = molecule_energy_densities(atoms, cols, clip_cte, ehf)
        return torch.where(dens.abs() > clip_cte, dens, torch.zeros((), dtype=dens.dtype, device=dens.device))

    def compute_coefficient_inputs(self, atoms, *args, **kwargs):
        if self.coefficient_inputs is None and self.nograd_coefficient_inputs is None:
            return None
        raise NotImplementedError("coefficient inputs are only supported by NeuralFunctional/DM21")

    def xc_energy(self, params, grid, coefficient_inputs, densities, clip_cte: float = CLIP, **kwargs):
        """functional.py:219-253 on given densities (device reduction, Kahan FP64)."""
        import ctypes
        coeffs = _const_row(self.apply(params, coefficient_inputs))
        dens = densities.contiguous()
        n_grid, n_cols = dens.shape
        w = engine.as_device_f64(grid.weights, dens.device)
        ws_bytes = ctypes.c_size_t()
        _lib.check(_lib.load().gdft_integrate_workspace_bytes(n_grid, ctypes.byref(ws_bytes)))
        ws = torch.empty(ws_bytes.value, dtype=torch.uint8, device=dens.device)
        out = torch.empty((), dtype=torch.float64, device=dens.device)
        carr = (ctypes.c_double * len(coeffs))(*coeffs)
        _lib.check(_lib.load().gdft_integrate(n_grid, n_cols, carr, len(coeffs), engine._ptr(dens), engine._ptr(w),
                                              float(clip_cte), engine._ptr(out), engine._ptr(ws), ws.numel(),
                                              engine._stream(dens.device)))
        return out

    def xc_energy_and_grads(self, params, atoms, clip_cte: float = CLIP):
        """(E_xc, dE_xc/d rdm1) through the fused device path (train.py:86-121)."""
        fn, ehf = self.spec(params, atoms, clip_cte)
        return atoms.resident().xc_energy_and_grads(atoms._rdm1(), fn, ehf, want_vxc=True)

    def xc_energy_and_potential(self, params, atoms, clip_cte: float = CLIP):
        """(E_xc, V_xc) of one device pass, E_xc differentiable in rdm1 (as the energies of the SCF
        loops and the orbital optimisers need); V_xc is a constant of the autograd graph."""
        fn, ehf = self.spec(params, atoms, clip_cte)
        rdm1 = atoms.rdm1 if isinstance(atoms.rdm1, torch.Tensor) and atoms.rdm1.requires_grad else atoms._rdm1()
        return _XcEnergyPotential.apply(rdm1, atoms.resident(), fn, ehf)

    def hf_density_gradient(self, params, atoms, ehf, clip_cte: float = CLIP):
        """dE_xc/d ehf (omega, spin, grid) through the densities, the gradient that
        HF_density_grad_2_Fock takes (molecule.py:598-603): the same for every
        (omega, spin) because the HF column is their sum (b3lyp_combine)."""
        cols = energy_density_columns(self.energy_densities) if self.energy_densities is not None else ()
        hf_cols = getattr(self.combine_densities, "_gdft_hf_cols", None) if self.combine_densities else None
        if hf_cols != (_lib.COL_HF,):
            raise NotImplementedError("the HF-density gradient is built for functionals whose HF column is "
                                      "the sum of ehf over omega and spin (b3lyp_combine)")
        if self.coefficient_inputs is not None or self.nograd_coefficient_inputs is not None:
            raise NotImplementedError("coefficient inputs are only supported by NeuralFunctional/DM21")
        coeffs = _const_row(self.coefficients(self, None))
        fn = engine.make_functional(cols + tuple(hf_cols), coeffs, clip_cte)
        _, _, g = atoms.resident().xc_energy_grads_hf(atoms._rdm1(), fn, ehf, want_vxc=False)
        return g[None, None, :].expand(ehf.shape[0], 2, g.shape[0]).contiguous()

    def hf_cinput_gradient(self, params, atoms, ehf, clip_cte: float = CLIP):
        """dE_xc/d ehf through the coefficient inputs: none for constant coefficients."""
        raise NotImplementedError("the functional's coefficients do not depend on HF inputs")

    def energy_xc_only(self, params, atoms, *args, **kwargs):
        fn, ehf = self.spec(params, atoms, kwargs.get("clip_cte", CLIP))
        if getattr(atoms, "is_solid", False):  # E_xc of the k-points (no autograd through a complex rdm1)
            return atoms.resident().xc_energy_and_grads(atoms._rdm1(), fn, ehf, want_vxc=False)[0]
        rdm1 = atoms.rdm1 if isinstance(atoms.rdm1, torch.Tensor) and atoms.rdm1.requires_grad else atoms._rdm1()
        return _XcEnergy.apply(rdm1, atoms.resident(), fn, ehf)

    def energy(self, params, atoms, *args, **kwargs):
        """functional.py:255-288."""
        e = self.energy_xc_only(params, atoms, *args, **kwargs)
        if self.is_xc:
            e = e + atoms.nonXC()
        return e


def _hf_cols(*cols):
    def deco(f):
        f._gdft_hf_cols = tuple(cols)
        return f

    return deco


@_hf_cols(_lib.COL_HF_W0, _lib.COL_HF_W1)
def dm21_combine_densities(densities, ehf):
    """functional.py:652-675: append sum over spin of ehf for each omega."""
    parts = [densities] + [ehf[i].sum(dim=0, keepdim=True).T for i in range(len(ehf))]
    return torch.cat(parts, dim=1)


def _uw_ranges(functional_type):
    """u_range / w_range of dm21_densities and densities (functional.py:575-585, 1089-1099).

    A dict {'u_range': ..., 'w_range': ...} follows the documented meaning
    (functional.py:548-556); the reference's own code binds the ranges only
    for a string and raises UnboundLocalError for a dict."""
    if isinstance(functional_type, str):
        if functional_type in ("LDA", "DM21"):
            return range(0, 1), range(0, 1)
        if functional_type == "GGA":
            return range(0, 2), range(0, 1)
        if functional_type == "MGGA":
            return range(0, 2), range(0, 2)
        raise ValueError(f"Functional type {functional_type} not recognized, must be one of LDA, GGA, MGGA.")
    if isinstance(functional_type, dict) and set(functional_type) == {"u_range", "w_range"}:
        u, w = list(functional_type["u_range"]), list(functional_type["w_range"])
        if not all(isinstance(k, int) and 0 <= k <= 15 for k in u + w):
            raise NotImplementedError("u_range / w_range powers must be integers in 0..15")
        return u, w
    raise ValueError(f"Functional type {functional_type} not recognized, must be one of LDA, GGA, MGGA "
                     "or a dict with u_range and w_range")


def _dm21_cols(functional_type="LDA"):
    u, w = _uw_ranges(functional_type)
    return tuple(_lib.COL_DM21_LDA if (i, j) == (0, 0) else _lib.col_dm21_uw(i, j) for i in u for j in w)


def _densities_cols(functional_type="LDA"):
    u, w = _uw_ranges(functional_type)
    ex = tuple(_lib.col_dens_x(s, i, j) for i in u for j in w for s in (0, 1))
    return ex + (_lib.COL_ZERO,) * (2 * len(u) * len(w))


def _check_cols(cols, fname):
    if len(cols) > _lib.MAX_COLS:
        raise NotImplementedError(f"{fname}: {len(cols)} columns; the device functional holds {_lib.MAX_COLS}")
    return cols


def dm21_densities(atoms, functional_type="LDA", clip_cte: float = CLIP, *_, **__):
    """functional.py:534-626: one column per (i, j) in u_range x w_range, sum over spin of
    2^(4/3 log rho + i log u + j log w), the (0, 0) column scaled to DM21's LDA exchange."""
    cols = _check_cols(_dm21_cols(functional_type), "dm21_densities")
    return molecule_energy_densities(atoms, cols, clip_cte)


dm21_densities._gdft_cols = (_lib.COL_DM21_LDA,)
dm21_densities._gdft_cols_of = _dm21_cols


def densities(atoms, functional_type="LDA", clip_cte: float = CLIP, *_, **__):
    """functional.py:1048-1202: per (i, j) the two spins' exchange terms 2^(4/3 log rho + i log u + j log w)
    (log 1/t = log tau - 5/3 log rho), then per (i, j) the two correlation features.  Those are
    where(round(e_PW92, int(log10(clip_cte))) > clip_cte, ..., 0) (:1188-1197): e_PW92 is negative and
    clip_cte positive, so they are zero for every input, with zero gradient."""
    cols = _check_cols(_densities_cols(functional_type), "densities")
    return molecule_energy_densities(atoms, cols, clip_cte)


densities._gdft_cols = _densities_cols("LDA")
densities._gdft_cols_of = _densities_cols


def dm21_combine_cinputs(cinputs, ehf):
    """functional.py:628-649."""
    return torch.cat([cinputs, ehf[:, 0].T, ehf[:, 1].T], dim=1)


def canonicalize_inputs(x):
    """functional.py:934-945."""
    x = torch.as_tensor(x)
    if x.ndim == 1:
        return x[:, None]
    if x.ndim == 0:
        raise ValueError("`features` has to be at least 1D array!")
    return x
