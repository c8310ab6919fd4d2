"""energy_predictor (train.py:34-218): (E, Fock) through the fused device path."""
from __future__ import annotations

from typing import Callable, Optional

from . import engine
from .functional import CLIP


def energy_predictor(functional, nlc_functional=None, clip_cte: float = CLIP, **kwargs) -> Callable:
    """train.py:34-218.

    ``predict(params, atoms) -> (E, F)``: E = E_xc + nonXC and
    F = abs_clip(1/2 (G + G^T)) with G = abs_clip(h1e + J + dE_xc/d rdm1)
    (train.py:147-163), plus the explicit HF Fock terms of ``densitygrads`` /
    ``coefficient_input_grads`` (train.py:165-213) computed from the
    molecule's chi tensor; as in the reference, a functional that has them
    raises ``ValueError`` when the molecule has no chi.
    """
    if nlc_functional is not None:
        raise NotImplementedError("dispersion (nlc) functionals are not part of the XC grid path")

    def predict(params, atoms, *args):
        needs_chi = functional.densitygrads is not None or functional.coefficient_input_grads is not None
        if getattr(atoms, "is_solid", False):
            # train.py:147-163 with a Solid: F = h1e + J + n_kpt dE_xc/d rdm1 (complex, jax.grad's
            # convention), clipped, (F + F^H)/2, clipped; hybrid terms are not available for solids.
            if needs_chi:
                atoms.select_HF_omegas(None)
            exc, vxc = functional.xc_energy_and_grads(params, atoms, clip_cte)
            r = atoms.resident()
            vj, enonxc = r.coulomb(atoms.rep_tensor, atoms._rdm1(), atoms.h1e, float(atoms.nuclear_repulsion),
                                   want_energy=True)
            return exc + enonxc, r.fock(atoms.h1e, vj, vxc, clip_cte)
        if needs_chi and getattr(atoms, "chi", None) is None:
            raise ValueError("Precomputed chi tensor has not been loaded.")
        exc, vxc = functional.xc_energy_and_grads(params, atoms, clip_cte)
        rdm1 = atoms._rdm1()
        vj, enonxc = engine.coulomb(atoms.rep_tensor, rdm1, atoms.h1e, float(atoms.nuclear_repulsion),
                                    want_energy=True)
        energy = exc + enonxc
        fock = engine.fock(atoms.h1e, vj, vxc, clip_cte)
        if needs_chi and _cached_library_hf_terms(functional, params, atoms):
            # The library's DM21 HF terms take dE_xc/d ehf from the network pass just made; they read
            # none of the densities, inputs or ehf that train.py:165-196 builds for other terms.
            if functional.densitygrads is not None:
                vxc_expl = functional.densitygrads(functional, params, atoms, None, None, None)
                fock = engine.fock_add_hf(fock, vxc_expl, clip_cte)
            if functional.coefficient_input_grads is not None:
                vxc_expl = functional.coefficient_input_grads(functional, params, atoms, None, None, None)
                fock = engine.fock_add_hf(fock, vxc_expl, clip_cte)
        elif needs_chi:
            # train.py:165-213: the explicit HF terms, each added as F + F^T and clipped.
            grad_densities = functional.energy_densities(atoms) if functional.energy_densities is not None else None
            nograd_densities = functional.nograd_densities(atoms) if functional.nograd_densities else None
            densities = grad_densities
            if grad_densities is not None and nograd_densities is not None:
                densities = functional.combine_densities(grad_densities, nograd_densities)
            grad_cinputs = functional.coefficient_inputs(atoms) if functional.coefficient_inputs else None
            nograd_cinputs = (functional.nograd_coefficient_inputs(atoms)
                              if functional.nograd_coefficient_inputs else None)
            cinputs = grad_cinputs
            if grad_cinputs is not None and nograd_cinputs is not None:
                cinputs = functional.combine_inputs(grad_cinputs, nograd_cinputs)
            if functional.densitygrads is not None:
                vxc_expl = functional.densitygrads(functional, params, atoms, nograd_densities, cinputs,
                                                   grad_densities)
                fock = engine.fock_add_hf(fock, vxc_expl, clip_cte)
            if functional.coefficient_input_grads is not None:
                vxc_expl = functional.coefficient_input_grads(functional, params, atoms, nograd_cinputs,
                                                              grad_cinputs, densities)
                fock = engine.fock_add_hf(fock, vxc_expl, clip_cte)
        return energy, fock

    return predict


def _cached_library_hf_terms(functional, params, atoms) -> bool:
    """True when every HF Fock term of ``functional`` is one of the library's DM21 terms (marked
    ``_gdft_reads_ehf_only``) and their dE_xc/d ehf is cached for this molecule, parameters and the
    clip they look it up with."""
    slots = [f for f in (functional.densitygrads, functional.coefficient_input_grads) if f is not None]
    if not slots or not all(getattr(f, "_gdft_reads_ehf_only", False) for f in slots):
        return False
    cached = getattr(functional, "_hf_cached", None)
    return cached is not None and cached(params, atoms, CLIP) is not None
