"""GB300-native XC grid path of Grad DFT.

The public names mirror ``grad_dft`` (grad_dft/__init__.py) for the XC path:
containers, density primitives, the Functional plugin API, the classical
functionals and ``energy_predictor``.  Compute runs in ``libgdft_xc.so``
(hand-written sm_103a CUDA behind a C ABI); there is no CPU fallback.
"""
from .molecule import Grid, Molecule, abs_clip, density, grad_density, lapl_density, kinetic_density
from .functional import (
    Functional,
    canonicalize_inputs,
    dm21_combine_cinputs,
    dm21_combine_densities,
    densities,
    dm21_densities,
    stack_densities,
)
from .popular_functionals import (
    B3LYP,
    B88,
    BLYP,
    LSDA,
    LYP,
    PW92,
    VWN,
    b3lyp_combine,
    b3lyp_exhf_densities,
    b88_density,
    lsda_density,
    lyp_density,
    pw92_densities,
    vwn_density,
)
from .train import energy_predictor
from .scf import (Diis, JittableDiis, diff_scf_loop, scf_loop, diff_simple_scf_loop, jitted_mol_orb_optimizer, mol_orb_optimizer,
                  non_scf_predictor, safe_eigh, safe_fock_solver, safe_general_eigh, simple_scf_loop)
from . import optim
from .basis import ShellBasis, eval_ao, molecule_from_basis
from . import chi
from .solid import KPointInfo, Solid
from .chi import generate_chi_tensor
from .neural import DM21, NeuralFunctional, dm21_coefficient_inputs, dm21_hfgrads_cinputs, dm21_hfgrads_densities

__all__ = [
    "Grid", "Molecule", "abs_clip", "density", "grad_density", "lapl_density", "kinetic_density",
    "Functional", "canonicalize_inputs", "dm21_combine_cinputs", "dm21_combine_densities", "dm21_densities",
    "densities", "stack_densities", "B3LYP", "B88", "BLYP", "LSDA", "LYP", "PW92", "VWN", "b3lyp_combine",
    "b3lyp_exhf_densities", "b88_density", "lsda_density", "lyp_density", "pw92_densities", "vwn_density",
    "energy_predictor", "DM21", "NeuralFunctional", "dm21_coefficient_inputs", "dm21_hfgrads_cinputs",
    "dm21_hfgrads_densities", "diff_simple_scf_loop", "diff_scf_loop", "JittableDiis", "safe_eigh",
    "safe_fock_solver", "safe_general_eigh", "ShellBasis", "eval_ao", "molecule_from_basis",
    "generate_chi_tensor", "Solid", "KPointInfo", "simple_scf_loop", "non_scf_predictor",
    "mol_orb_optimizer", "jitted_mol_orb_optimizer", "optim", "scf_loop", "Diis",
]
