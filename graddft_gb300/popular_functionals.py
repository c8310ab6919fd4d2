"""Classical functionals with the reference's names (popular_functionals.py:271-393)."""
from __future__ import annotations

import torch

from . import _lib
from .functional import CLIP, Functional, _hf_cols, molecule_energy_densities, stack_densities, tag_columns


@tag_columns(_lib.COL_LSDA)
def lsda_density(molecule, clip_cte: float = CLIP, *_, **__):
    """popular_functionals.py:271-275."""
    return molecule_energy_densities(molecule, (_lib.COL_LSDA,), clip_cte)


@tag_columns(_lib.COL_LSDA, _lib.COL_B88)
def b88_density(molecule, clip_cte: float = CLIP, *_, **__):
    """popular_functionals.py:277-284: columns (lsda_x_e, b88_x_e)."""
    return molecule_energy_densities(molecule, (_lib.COL_LSDA, _lib.COL_B88), clip_cte)


@tag_columns(_lib.COL_VWN)
def vwn_density(molecule, clip_cte: float = CLIP, *_, **__):
    """popular_functionals.py:286-290."""
    return molecule_energy_densities(molecule, (_lib.COL_VWN,), clip_cte)


@tag_columns(_lib.COL_PW92)
def pw92_densities(molecule, clip_cte: float = CLIP, *_, **__):
    """popular_functionals.py:292-296."""
    return molecule_energy_densities(molecule, (_lib.COL_PW92,), clip_cte)


@tag_columns(_lib.COL_LYP)
def lyp_density(molecule, clip_cte: float = CLIP, *_, **__):
    """popular_functionals.py:298-304."""
    return molecule_energy_densities(molecule, (_lib.COL_LYP,), clip_cte)


@tag_columns(_lib.COL_LSDA, _lib.COL_B88, _lib.COL_VWN, _lib.COL_LYP)
def b3lyp_exhf_densities(molecule, clip_cte: float = CLIP, *_, **__):
    """popular_functionals.py:306-326: (lsda, b88, vwn, lyp)."""
    return molecule_energy_densities(molecule, (_lib.COL_LSDA, _lib.COL_B88, _lib.COL_VWN, _lib.COL_LYP), clip_cte)


@_hf_cols(_lib.COL_HF)
def b3lyp_combine(features, ehf):
    """popular_functionals.py:328-334: append sum_{omega, spin} ehf."""
    return torch.cat([features, ehf.sum(dim=(0, 1))[:, None]], dim=1)


def b3lyp_coefficients(instance, *args):
    """popular_functionals.py:336-343."""
    a0, ax, ac = 0.2, 0.72, 0.81
    return torch.tensor([[1 - a0, ax, 1 - ac, ac, a0]], dtype=torch.float64)


def b3lyp_nograd_densities(molecule, *_, **__):
    """popular_functionals.py:345-350."""
    return molecule.HF_energy_density([0.0])


def b3lyp_hfgrads(functional, params, molecule, ehf, cinputs, densities_wout_hf, omegas=(0.0,)):
    """popular_functionals.py:352-372: the explicit HF Fock term, summed over omega (needs chi)."""
    vxc_hf = molecule.HF_density_grad_2_Fock(functional, params, omegas, ehf, cinputs, densities_wout_hf)
    return vxc_hf.sum(dim=0)


def _one(self, *_):
    return torch.tensor([[1.0]], dtype=torch.float64)


LSDA = Functional(coefficients=_one, energy_densities=lsda_density)
B88 = Functional(coefficients=_one, energy_densities=b88_density)
VWN = Functional(coefficients=_one, energy_densities=vwn_density)
LYP = Functional(coefficients=_one, energy_densities=lyp_density, exchange_mask=torch.tensor([]))
B3LYP = Functional(
    coefficients=b3lyp_coefficients,
    energy_densities=b3lyp_exhf_densities,
    nograd_densities=b3lyp_nograd_densities,
    densitygrads=b3lyp_hfgrads,
    combine_densities=b3lyp_combine,
    exchange_mask=torch.tensor([1, 1, 0, 0, 1]),
)
PW92 = Functional(coefficients=_one, energy_densities=pw92_densities)
# B88 exchange + LYP correlation with unit coefficients (lsda_x + b88 correction + lyp).
BLYP = Functional(coefficients=_one, energy_densities=stack_densities(b88_density, lyp_density))
