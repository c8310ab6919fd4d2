"""energy_predictor (train.py:34-218): (E, Fock) through the fused device path."""
from __future__ import annotations

from typing import Callable, Optional

from . import engine
from .functional import CLIP


def energy_predictor(functional, nlc_functional=None, clip_cte: float = CLIP, **kwargs) -> Callable:
    """train.py:34-218.

    ``predict(params, atoms) -> (E, F)``: E = E_xc + nonXC and
    F = abs_clip(1/2 (G + G^T)) with G = abs_clip(h1e + J + dE_xc/d rdm1)
    (train.py:147-163).  The explicit HF Fock terms (train.py:200-213) need a
    chi tensor: as in the reference, a functional with ``densitygrads`` or
    ``coefficient_input_grads`` raises ``ValueError`` when the molecule has none.
    """
    if nlc_functional is not None:
        raise NotImplementedError("dispersion (nlc) functionals are not part of the XC grid path")

    def predict(params, atoms, *args):
        needs_chi = functional.densitygrads is not None or functional.coefficient_input_grads is not None
        if needs_chi and getattr(atoms, "chi", None) is None:
            raise ValueError("Precomputed chi tensor has not been loaded.")
        exc, vxc = functional.xc_energy_and_grads(params, atoms, clip_cte)
        rdm1 = atoms._rdm1()
        vj, enonxc = engine.coulomb(atoms.rep_tensor, rdm1, atoms.h1e, float(atoms.nuclear_repulsion),
                                    want_energy=True)
        energy = exc + enonxc
        fock = engine.fock(atoms.h1e, vj, vxc, clip_cte)
        if needs_chi:
            raise NotImplementedError("the chi-based HF Fock contributions are not built in this version")
        return energy, fock

    return predict
