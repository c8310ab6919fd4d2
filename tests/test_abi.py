"""The C-ABI library builds, loads and exports every symbol include/gdft.h declares (no GPU needed)."""
import ctypes
import os
import re

from conftest import ROOT


def _declared():
    src = open(os.path.join(ROOT, "include", "gdft.h")).read()
    return sorted(set(re.findall(r"^(?:int|const char \*)\s*(gdft_[a-z0-9_]+)\(", src, re.M)))


def test_header_and_binding_agree():
    from graddft_gb300 import _lib

    assert sorted(_lib.EXPORTS) == _declared()


def test_library_exports_all_symbols(built_lib):
    lib = ctypes.CDLL(built_lib)
    for name in _declared():
        assert hasattr(lib, name), name


def test_host_only_calls(built_lib):
    from graddft_gb300 import _lib

    lib = _lib.load(built_lib)
    assert lib.gdft_abi_version() == 1
    nbytes = ctypes.c_size_t()
    assert lib.gdft_molecule_bytes(1000, 40, _lib.GDFT_FP64, ctypes.byref(nbytes)) == 0
    # five FP64 planes of 1024 x 64 plus the weights
    assert nbytes.value >= 5 * 1024 * 64 * 8 + 1024 * 8
    assert lib.gdft_molecule_bytes(0, 40, _lib.GDFT_FP64, ctypes.byref(nbytes)) == _lib.GDFT_ERR_INVALID
    assert b"positive" in lib.gdft_last_error()
    mol = _lib.GdftMolecule()
    # a buffer that is too small is rejected before any device work
    assert lib.gdft_molecule_init(ctypes.byref(mol), 1000, 40, 0, ctypes.c_void_p(256), 16) == _lib.GDFT_ERR_WORKSPACE
    # misaligned buffer
    assert lib.gdft_molecule_init(ctypes.byref(mol), 1000, 40, 0, ctypes.c_void_p(8), 1 << 30) == _lib.GDFT_ERR_ALIGNMENT
    assert lib.gdft_fock(0, None, None, None, 1e-30, None, None) == _lib.GDFT_ERR_INVALID


def test_functional_dispatch_host_side():
    import pytest
    import torch

    import graddft_gb300 as g
    from graddft_gb300 import _lib, engine

    fn = engine.make_functional([_lib.COL_LSDA, _lib.COL_B88], [1.0])
    assert fn.n_cols == 2 and fn.n_coeffs == 1 and fn.cols[1] == _lib.COL_B88
    with pytest.raises(ValueError):
        engine.make_functional([], [1.0])
    with pytest.raises(ValueError):
        engine.make_functional([0, 1, 2], [1.0, 2.0])
    # Known plugin callables map to kernel columns; the spec needs no device.
    assert g.B88._columns(None) == ((_lib.COL_LSDA, _lib.COL_B88), None)
    assert g.BLYP._columns(None)[0] == (_lib.COL_LSDA, _lib.COL_B88, _lib.COL_LYP)
    # An unknown energy-density callable has no kernel: it raises instead of falling back.
    custom = g.Functional(coefficients=lambda self, *_: torch.tensor([[1.0]]), energy_densities=lambda m: None)
    with pytest.raises(NotImplementedError):
        custom._columns(None)
