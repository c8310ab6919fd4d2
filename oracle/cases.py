"""Seeded inputs of fixture cases that are regenerated instead of stored (test infrastructure).

The B3LYP case at n_ao = 43 stands in for the reference's config-1 molecule
(H2O / def2-TZVP, unrestricted B3LYP on a converged density matrix), whose
PySCF inputs are not available here: the same number of AOs, a seeded s/p/d
basis on a 4,096-point grid, a fixed density matrix and a stand-in chi tensor
for the exact-exchange column (omega 0).  tests/golden/make_golden.py stores
only what the reference computes from these inputs.
"""
from __future__ import annotations

import numpy as np

from graddft_gb300 import synthetic

from .ao_numpy import eval_ao_planes

B3LYP43 = dict(n_grid=4096, n_ao=43, n_occ=5, seed=43, box_angstrom=6.0, centre_box_angstrom=4.0, chi_seed=44)


def b3lyp43_inputs():
    """(workload, ao, grad_ao, grad2_ao, chi (grid, 1, 2, 43), omegas [0.0])."""
    c = B3LYP43
    wl = synthetic.make_workload(c["n_grid"], c["n_ao"], c["n_occ"], c["seed"], box_angstrom=c["box_angstrom"],
                                 centre_box_angstrom=c["centre_box_angstrom"])
    ao, g1, g2 = eval_ao_planes(wl.basis, wl.coords)
    chi = synthetic.make_chi(ao, wl.rdm1, n_omega=1, seed=c["chi_seed"])
    return wl, ao, g1, g2, chi, np.array([0.0])
