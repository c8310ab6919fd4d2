"""The chi tensor of the exact-exchange terms, built on the device.

``generate_chi_tensor`` follows ``interface/pyscf.py:1067-1126``:

    chi[r, w, s, a] = sum_(b,d) D_s[b, d] phi_b(r) nu^(omega_w)_(d a)(r)

with the range-separated integrals of ``_evaluate_nu`` / ``_nu_chunk``
(``external/_hf_density.py:17-120``, PySCF's ``int1e_grids``):

    nu_(d a)(r) = int phi_d(r') phi_a(r') erf(omega |r - r'|) / |r - r'| dr'   (omega = 0: 1/|r - r'|).

The integrals run in ``libgdft_xc.so`` (McMurchie-Davidson, FP64) for shells
up to l = 3; chi for a chunk of grid points is contracted from the chunk's
integrals without leaving the device.
"""
from __future__ import annotations

import ctypes
from typing import Sequence

import torch

from . import _lib, engine
from .basis import ShellBasis

F64 = torch.float64
MAX_OMEGA = 8


def _as_basis(mol) -> ShellBasis:
    if isinstance(mol, ShellBasis):
        return mol
    if hasattr(mol, "_bas") and hasattr(mol, "_env"):
        return ShellBasis.from_pyscf(mol)
    raise TypeError("mol must be a ShellBasis or a PySCF Mole (its _atm/_bas/_env arrays are read)")


def _workspace(desc, chunk: int, dev) -> torch.Tensor:
    nbytes = ctypes.c_size_t()
    _lib.check(_lib.load().gdft_nu_workspace_bytes(ctypes.byref(desc), int(chunk), ctypes.byref(nbytes)))
    return torch.empty(max(nbytes.value, 256), dtype=torch.uint8, device=dev)


def nu_integrals(mol, coords, omega: float, device=None) -> torch.Tensor:
    """_evaluate_nu (external/_hf_density.py:56-70): (grid, ao, ao)."""
    if omega < 0:
        raise ValueError("Range-separated parameter omega must be non-negative!")
    dev = engine.require_cuda(device)
    basis = _as_basis(mol)
    coords = engine.as_device_f64(coords, dev)
    if coords.ndim != 2 or coords.shape[1] != 3:
        raise ValueError(f"coords must be (grid, 3), got {tuple(coords.shape)}")
    desc, _keep = basis.device_desc(dev)
    n = desc.n_ao
    nu = torch.empty((coords.shape[0], n, n), dtype=F64, device=dev)
    ws = _workspace(desc, 0, dev)
    _lib.check(_lib.load().gdft_nu_integrals(ctypes.byref(desc), engine._ptr(coords), coords.shape[0], float(omega),
                                             engine._ptr(nu), engine._ptr(ws), ws.numel(), engine._stream(dev)))
    return nu


def generate_chi_tensor(rdm1, ao, grid_coords, mol, omegas: Sequence[float], chunk_size: int = 1024,
                        precision=None, device=None) -> torch.Tensor:
    """interface/pyscf.py:1067-1126: chi (grid, omega, spin, ao).

    ``mol`` is a ``ShellBasis`` or a PySCF ``Mole``; ``precision`` is accepted
    for signature compatibility (the contraction is FP64).  ``chunk_size``
    bounds the integrals held at once (n_ao^2 * chunk_size doubles), as in the
    reference.
    """
    del precision
    omegas = [float(w) for w in omegas]
    dev = engine.require_cuda(device)
    if not omegas:
        return torch.zeros((0,), dtype=F64, device=dev)
    if any(w < 0 for w in omegas):
        raise ValueError("Range-separated parameter omega must be non-negative!")
    if len(omegas) > MAX_OMEGA:  # one library call takes up to MAX_OMEGA
        return torch.cat([generate_chi_tensor(rdm1, ao, grid_coords, mol, omegas[i:i + MAX_OMEGA], chunk_size,
                                              device=dev) for i in range(0, len(omegas), MAX_OMEGA)], dim=1)
    basis = _as_basis(mol)
    ao = engine.as_device_f64(ao, dev)
    rdm1 = engine.as_device_f64(rdm1, dev)
    coords = engine.as_device_f64(grid_coords, dev)
    desc, _keep = basis.device_desc(dev)
    n_grid, n = ao.shape[0], desc.n_ao
    if ao.shape != (n_grid, n) or coords.shape != (n_grid, 3):
        raise ValueError(f"ao {tuple(ao.shape)} / coords {tuple(coords.shape)} do not match ({n_grid}, {n}) / (grid, 3)")
    if rdm1.shape != (2, n, n):
        raise ValueError(f"rdm1 must be (2, {n}, {n}), got {tuple(rdm1.shape)}")
    chunk = max(1, min(int(chunk_size), n_grid))
    ws = _workspace(desc, chunk, dev)
    chi = torch.empty((n_grid, len(omegas), 2, n), dtype=F64, device=dev)
    h_om = (ctypes.c_double * len(omegas))(*omegas)
    _lib.check(_lib.load().gdft_chi(ctypes.byref(desc), engine._ptr(coords), engine._ptr(ao), engine._ptr(rdm1),
                                    n_grid, h_om, len(omegas), chunk, engine._ptr(chi), engine._ptr(ws), ws.numel(),
                                    engine._stream(dev)))
    return chi
