"""ctypes binding of libgdft_xc.so (the C ABI declared in include/gdft.h).

The library is built in-tree by ``graddft_gb300.build``.  There is no CPU or
eager-PyTorch fallback: if the shared library is missing, importing the
compute path raises immediately.
"""
from __future__ import annotations

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libgdft_xc.so")

GDFT_OK = 0
GDFT_ERR_INVALID = 1
GDFT_ERR_ALIGNMENT = 2
GDFT_ERR_WORKSPACE = 3
GDFT_ERR_CUDA = 4
GDFT_ERR_DEVICE = 5
GDFT_ERR_UNSUPPORTED = 6

GDFT_WAIT_EXPIRY_PROBE = 99

GDFT_FP64 = 0
GDFT_TF32X3 = 1

ABI_VERSION = 2

COL_LSDA, COL_B88, COL_VWN, COL_LYP, COL_PW92, COL_HF, COL_DM21_LDA, COL_HF_W0, COL_HF_W1, COL_ZERO = range(10)
MAX_COLS = 16


def col_dm21_uw(i: int, j: int) -> int:
    """GDFT_COL_DM21_UW(i, j): dm21_densities' u^i w^j term summed over spin (functional.py:616-624)."""
    return 0x100 | (i << 4) | j


def col_dens_x(spin: int, i: int, j: int) -> int:
    """GDFT_COL_DENS_X(s, i, j): densities()' exchange term u^i w^j of one spin (functional.py:1130-1134)."""
    return 0x200 | (spin << 8) | (i << 4) | j

# Every symbol include/gdft.h declares.
EXPORTS = (
    "gdft_abi_version", "gdft_last_error", "gdft_molecule_bytes", "gdft_molecule_init", "gdft_molecule_load",
    "gdft_molecule_eval_basis", "gdft_eval_ao", "gdft_molecule_eval_shells", "gdft_nu_workspace_bytes",
    "gdft_nu_integrals", "gdft_chi", "gdft_kpoint_workspace_bytes", "gdft_kpoint_density",
    "gdft_kpoint_xc_energy_and_grads", "gdft_kpoint_coulomb", "gdft_kpoint_fock", "gdft_workspace_bytes",
    "gdft_density", "gdft_xc_energy_and_grads",
    "gdft_energy_densities", "gdft_vxc_from_potentials", "gdft_integrate", "gdft_integrate_workspace_bytes", "gdft_integrate_noalloc", "gdft_fock", "gdft_coulomb",
    "gdft_profile_enable", "gdft_profile_reset", "gdft_profile_read", "gdft_device_status", "gdft_selftest_umma",
    "gdft_umma_probe", "gdft_network_param_count", "gdft_neural_workspace_bytes",
    "gdft_neural_xc_energy_and_grads", "gdft_neural_inputs", "gdft_network_apply_workspace_bytes",
    "gdft_network_apply", "gdft_neural_hvp_workspace_bytes", "gdft_neural_xc_hvp", "gdft_tc_gemm_probe",
    "gdft_tc_gemm3_probe", "gdft_neural_batch_workspace_bytes", "gdft_neural_batch_xc", "gdft_neural_batch_status",
    "gdft_xc_energy_grads_hf", "gdft_hf_workspace_bytes", "gdft_hf_energy_density", "gdft_hf_fock",
    "gdft_fock_add_hf", "gdft_neural_xc_hf_grads", "gdft_hf_workspace_bytes_form", "gdft_hf_energy_density_form",
    "gdft_hf_fock_form", "gdft_hf_device_status", "gdft_selftest_wait_expiry", "gdft_chunked_workspace_bytes",
    "gdft_xc_energy_and_grads_chunked", "gdft_neural_xc_energy_and_grads_chunked", "gdft_chunked_status",
)
STAGE_AO, STAGE_DENSITY, STAGE_POINT, STAGE_VXC, STAGE_REDUCE, STAGE_MLP = range(6)


class GdftFunctional(ctypes.Structure):
    _fields_ = [
        ("n_cols", ctypes.c_int32),
        ("cols", ctypes.c_int32 * MAX_COLS),
        ("n_coeffs", ctypes.c_int32),
        ("coeffs", ctypes.c_double * MAX_COLS),
        ("clip", ctypes.c_double),
    ]


class GdftMolecule(ctypes.Structure):
    _fields_ = [
        ("n_grid", ctypes.c_int64),
        ("n_grid_pad", ctypes.c_int64),
        ("n_ao", ctypes.c_int32),
        ("ld", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("buffer", ctypes.c_void_p),
        ("buffer_bytes", ctypes.c_size_t),
    ]


class GdftNetwork(ctypes.Structure):
    _fields_ = [
        ("n_in", ctypes.c_int32),
        ("width", ctypes.c_int32),
        ("n_layers", ctypes.c_int32),
        ("n_out", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("squash_offset", ctypes.c_double),
        ("sigmoid_scale", ctypes.c_double),
        ("ln_eps", ctypes.c_double),
        ("clip", ctypes.c_double),
    ]


_lib = None
_lock = threading.Lock()

P = ctypes.c_void_p
I32, I64, SZ, D = ctypes.c_int32, ctypes.c_int64, ctypes.c_size_t, ctypes.c_double
class GdftBasis(ctypes.Structure):
    _fields_ = [
        ("n_shell", ctypes.c_int32),
        ("n_ao", ctypes.c_int32),
        ("n_prim", ctypes.c_int64),
        ("n_coef", ctypes.c_int64),
        ("n_trans", ctypes.c_int64),
        ("d_shell", ctypes.c_void_p),
        ("d_centre", ctypes.c_void_p),
        ("d_exp", ctypes.c_void_p),
        ("d_coef", ctypes.c_void_p),
        ("d_ao", ctypes.c_void_p),
        ("d_trans", ctypes.c_void_p),
    ]


PMOL = ctypes.POINTER(GdftMolecule)
PBAS = ctypes.POINTER(GdftBasis)
PFN = ctypes.POINTER(GdftFunctional)
PNET = ctypes.POINTER(GdftNetwork)

_SIGS = {
    "gdft_abi_version": ([], ctypes.c_int),
    "gdft_last_error": ([], ctypes.c_char_p),
    "gdft_molecule_bytes": ([I64, I32, I32, ctypes.POINTER(SZ)], ctypes.c_int),
    "gdft_molecule_init": ([PMOL, I64, I32, I32, P, SZ], ctypes.c_int),
    "gdft_molecule_load": ([PMOL, P, P, P, P, P], ctypes.c_int),
    "gdft_molecule_eval_basis": ([PMOL, P, P, P, P], ctypes.c_int),
    "gdft_eval_ao": ([PBAS, P, I64, I32, P, P, P, P], ctypes.c_int),
    "gdft_molecule_eval_shells": ([PMOL, PBAS, P, P, P], ctypes.c_int),
    "gdft_nu_workspace_bytes": ([PBAS, I64, ctypes.POINTER(SZ)], ctypes.c_int),
    "gdft_kpoint_workspace_bytes": ([PMOL, I32, ctypes.POINTER(SZ)], ctypes.c_int),
    "gdft_kpoint_coulomb": ([I32, I32, P, P, P, P, D, P, P, P], ctypes.c_int),
    "gdft_kpoint_fock": ([I32, I32, P, P, P, D, P, P], ctypes.c_int),
    "gdft_kpoint_density": ([PMOL, I32, P, ctypes.POINTER(ctypes.c_double), P, P, P, P, P, SZ, P], ctypes.c_int),
    "gdft_kpoint_xc_energy_and_grads": ([PMOL, I32, P, ctypes.POINTER(ctypes.c_double), PFN, P, P, P, SZ, P],
                                        ctypes.c_int),
    "gdft_nu_integrals": ([PBAS, P, I64, ctypes.c_double, P, P, SZ, P], ctypes.c_int),
    "gdft_chi": ([PBAS, P, P, P, I64, ctypes.POINTER(ctypes.c_double), I32, I64, P, P, SZ, P], ctypes.c_int),
    "gdft_workspace_bytes": ([PMOL, ctypes.POINTER(SZ)], ctypes.c_int),
    "gdft_density": ([PMOL, P, P, P, P, P, P, SZ, P], ctypes.c_int),
    "gdft_xc_energy_and_grads": ([PMOL, P, PFN, P, I32, P, P, P, SZ, P], ctypes.c_int),
    "gdft_xc_energy_grads_hf": ([PMOL, P, PFN, P, I32, P, P, P, P, SZ, P], ctypes.c_int),
    "gdft_hf_workspace_bytes": ([I64, I32, I32, ctypes.POINTER(SZ)], ctypes.c_int),
    "gdft_hf_energy_density": ([P, P, P, I64, I32, I32, P, P, SZ, P], ctypes.c_int),
    "gdft_hf_fock": ([P, P, P, I64, I32, I32, P, P, SZ, P], ctypes.c_int),
    "gdft_fock_add_hf": ([P, P, I32, D, P], ctypes.c_int),
    "gdft_hf_workspace_bytes_form": ([I64, I32, I32, I32, ctypes.POINTER(SZ)], ctypes.c_int),
    "gdft_hf_energy_density_form": ([P, P, P, I64, I32, I32, I32, P, P, SZ, P], ctypes.c_int),
    "gdft_hf_fock_form": ([P, P, P, I64, I32, I32, I32, P, P, SZ, P], ctypes.c_int),
    "gdft_hf_device_status": ([P, SZ, ctypes.POINTER(I32), P], ctypes.c_int),
    "gdft_neural_xc_hf_grads": ([PMOL, P, PNET, P, P, P, P, P, P, P, SZ, P], ctypes.c_int),
    "gdft_energy_densities": ([PMOL, P, PFN, P, I32, P, P, SZ, P], ctypes.c_int),
    "gdft_vxc_from_potentials": ([PMOL, P, P, P, SZ, P], ctypes.c_int),
    "gdft_integrate": ([I64, I32, P, I32, P, P, D, P, P, SZ, P], ctypes.c_int),
    "gdft_integrate_workspace_bytes": ([I64, ctypes.POINTER(SZ)], ctypes.c_int),
    "gdft_integrate_noalloc": ([I64, I32, P, I32, P, P, D, P, P], ctypes.c_int),
    "gdft_fock": ([I32, P, P, P, D, P, P], ctypes.c_int),
    "gdft_coulomb": ([I32, P, P, P, D, P, P, P], ctypes.c_int),
    "gdft_device_status": ([PMOL, P, SZ, ctypes.POINTER(I32), P], ctypes.c_int),
    "gdft_selftest_wait_expiry": ([PMOL, P, SZ, I32, P], ctypes.c_int),
    "gdft_chunked_workspace_bytes": ([I32, I64, I32, PNET, ctypes.POINTER(SZ)], ctypes.c_int),
    "gdft_xc_energy_and_grads_chunked": ([PBAS, P, I32, P, P, I64, I64, I32, P, PFN, P, I32, P, P, P, SZ, P],
                                         ctypes.c_int),
    "gdft_neural_xc_energy_and_grads_chunked": ([PBAS, P, I32, P, P, I64, I64, I32, P, PNET, P, P, P, P, P, P, SZ,
                                                 P], ctypes.c_int),
    "gdft_chunked_status": ([P, SZ, ctypes.POINTER(I32), P], ctypes.c_int),
    "gdft_selftest_umma": ([ctypes.POINTER(D)], ctypes.c_int),
    "gdft_umma_probe": ([P, P, P], ctypes.c_int),
    "gdft_network_param_count": ([PNET, ctypes.POINTER(SZ)], ctypes.c_int),
    "gdft_neural_workspace_bytes": ([PMOL, PNET, ctypes.POINTER(SZ)], ctypes.c_int),
    "gdft_neural_xc_energy_and_grads": ([PMOL, P, PNET, P, P, P, P, P, P, SZ, P], ctypes.c_int),
    "gdft_neural_inputs": ([PMOL, P, PNET, P, P, P, P, SZ, P], ctypes.c_int),
    "gdft_network_apply_workspace_bytes": ([PNET, I64, ctypes.POINTER(SZ)], ctypes.c_int),
    "gdft_network_apply": ([PNET, P, I64, P, P, P, SZ, P], ctypes.c_int),
    "gdft_neural_hvp_workspace_bytes": ([PMOL, PNET, ctypes.POINTER(SZ)], ctypes.c_int),
    "gdft_neural_xc_hvp": ([PMOL, P, PNET, P, P, P, P, P, P, P, SZ, P], ctypes.c_int),
    "gdft_tc_gemm_probe": ([I32, I32, I32, I32, P, P, P], ctypes.c_int),
    "gdft_tc_gemm3_probe": ([I32, I32, I32, I32, P, P, P], ctypes.c_int),
    "gdft_neural_batch_workspace_bytes": ([I32, P, PNET, ctypes.POINTER(SZ)], ctypes.c_int),
    "gdft_neural_batch_xc": ([I32, P, P, P, PNET, P, P, P, P, P, P, P, SZ, P], ctypes.c_int),
    "gdft_neural_batch_status": ([P, SZ, ctypes.POINTER(I32), P], ctypes.c_int),
    "gdft_profile_enable": ([I32], ctypes.c_int),
    "gdft_profile_reset": ([], ctypes.c_int),
    "gdft_profile_read": ([I32, ctypes.POINTER(D), ctypes.POINTER(I64)], ctypes.c_int),
}


def load(path: str | None = None):
    """Load libgdft_xc.so and declare the C signatures (raises if it is missing)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = path or LIB_PATH
        if not os.path.exists(path):
            raise ImportError(
                f"libgdft_xc.so not found at {path}; build it with `python -m graddft_gb300.build` "
                "(the XC path has no CPU fallback)")
        lib = ctypes.CDLL(path)
        for name, (args, res) in _SIGS.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        if lib.gdft_abi_version() != ABI_VERSION:
            raise ImportError("libgdft_xc.so ABI version mismatch")
        _lib = lib
        return lib


class GdftError(RuntimeError):
    pass


def check(rc: int) -> None:
    if rc == GDFT_OK:
        return
    msg = load().gdft_last_error().decode(errors="replace")
    if rc in (GDFT_ERR_INVALID, GDFT_ERR_WORKSPACE):
        raise ValueError(msg)
    if rc == GDFT_ERR_ALIGNMENT:
        raise TypeError(msg)
    if rc == GDFT_ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    raise GdftError(msg)
