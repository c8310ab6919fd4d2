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
    assert lib.gdft_abi_version() == _lib.ABI_VERSION == 2
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


def test_network_layout_host_side(built_lib):
    """The flat DM21 parameter layout agrees between the library and the Python packing."""
    import numpy as np
    import pytest

    from graddft_gb300 import _lib, engine, synthetic

    lib = _lib.load(built_lib)
    for layers, width in ((6, 256), (2, 64), (0, 32)):
        net = engine.Network(n_layers=layers, width=width)
        n = ctypes.c_size_t()
        assert lib.gdft_network_param_count(ctypes.byref(net.desc), ctypes.byref(n)) == 0
        assert n.value == net.n_params
    net = engine.Network()
    assert net.n_params == 11 * 256 + 256 + 6 * (256 * 256 + 3 * 256) + 256 * 3 + 3
    params = synthetic.glorot_params(seed=7)
    flat = net.flatten(params, "cpu")
    assert flat.shape == (net.n_params,)
    back = net.unflatten(flat)
    for mod, d in params["params"].items():
        for leaf, v in d.items():
            np.testing.assert_array_equal(back["params"][mod][leaf].numpy(), v)
    # Dense_0 kernel first, head bias last (the order include/gdft.h documents).
    np.testing.assert_array_equal(flat[:5].numpy(), params["params"]["Dense_0"]["kernel"].reshape(-1)[:5])
    np.testing.assert_array_equal(flat[-3:].numpy(), params["params"]["Dense_7"]["bias"])
    bad = engine.Network(width=100)
    assert lib.gdft_network_param_count(ctypes.byref(bad.desc), ctypes.byref(n)) == _lib.GDFT_ERR_INVALID
    wrong = engine.Network(n_in=7)
    assert lib.gdft_network_param_count(ctypes.byref(wrong.desc), ctypes.byref(n)) == _lib.GDFT_ERR_INVALID
    with pytest.raises(ValueError):
        net.flatten({"params": {"Dense_0": params["params"]["Dense_0"]}}, "cpu")


def test_host_only_argument_checks_new_entries(built_lib):
    """Basis, chi and k-point entries reject bad arguments before any device work."""
    from graddft_gb300 import _lib

    lib = _lib.load(built_lib)
    nbytes = ctypes.c_size_t()
    assert lib.gdft_eval_ao(None, None, 10, 1, None, None, None, None) == _lib.GDFT_ERR_INVALID
    assert lib.gdft_molecule_eval_shells(None, None, None, None, None) == _lib.GDFT_ERR_INVALID
    assert lib.gdft_nu_workspace_bytes(None, 0, ctypes.byref(nbytes)) == _lib.GDFT_ERR_INVALID
    assert lib.gdft_nu_integrals(None, None, 10, 0.0, None, None, 0, None) == _lib.GDFT_ERR_INVALID
    assert lib.gdft_chi(None, None, None, None, 10, None, 1, 8, None, None, 0, None) == _lib.GDFT_ERR_INVALID
    assert lib.gdft_kpoint_workspace_bytes(None, 1, ctypes.byref(nbytes)) == _lib.GDFT_ERR_INVALID
    assert lib.gdft_kpoint_fock(0, 4, None, None, None, 1e-30, None, None) == _lib.GDFT_ERR_INVALID
    assert lib.gdft_kpoint_coulomb(0, 4, None, None, None, None, 0.0, None, None, None) == _lib.GDFT_ERR_INVALID
    basis = _lib.GdftBasis()  # empty tables
    assert lib.gdft_eval_ao(ctypes.byref(basis), None, 10, 1, None, None, None, None) == _lib.GDFT_ERR_INVALID
    assert b"basis" in lib.gdft_last_error()


def test_host_only_checks_exchange_forms(built_lib):
    """The form-taking exchange entries: workspace sizes per form, unknown forms, missing pointers."""
    from graddft_gb300 import _lib

    lib = _lib.load(built_lib)
    fp64, mixed = ctypes.c_size_t(), ctypes.c_size_t()
    assert lib.gdft_hf_workspace_bytes_form(4099, 37, 2, _lib.GDFT_FP64, ctypes.byref(fp64)) == _lib.GDFT_OK
    legacy = ctypes.c_size_t()
    assert lib.gdft_hf_workspace_bytes(4099, 37, 2, ctypes.byref(legacy)) == _lib.GDFT_OK
    assert legacy.value == fp64.value
    assert lib.gdft_hf_workspace_bytes_form(4099, 37, 2, _lib.GDFT_TF32X3, ctypes.byref(mixed)) == _lib.GDFT_OK
    # error word + the larger of (ao sets, D sets, X) and (ao^T sets, B sets, split partials)
    set3, a256 = 3 * 128 * 32 * 4, (lambda x: (x + 255) // 256 * 256)
    energy = a256(33 * 2 * set3) + a256(1 * 2 * set3) + a256(4099 * 74 * 8)
    rch = (4099 + 31) // 32
    fock = a256(rch * set3) + a256(rch * set3) + a256(rch * 37 * 74 * 8)  # one split per K chunk here
    assert mixed.value == 256 + max(energy, fock)
    assert lib.gdft_hf_workspace_bytes_form(4099, 37, 2, 7, ctypes.byref(mixed)) == _lib.GDFT_ERR_INVALID
    assert lib.gdft_hf_energy_density_form(None, None, None, 10, 4, 1, _lib.GDFT_TF32X3, None, None, 0,
                                           None) == _lib.GDFT_ERR_INVALID
    assert lib.gdft_hf_fock_form(None, None, None, 10, 4, 1, 9, None, None, 0, None) == _lib.GDFT_ERR_INVALID
    assert b"form" in lib.gdft_last_error()
    status = ctypes.c_int32()
    assert lib.gdft_hf_device_status(None, 0, ctypes.byref(status), None) == _lib.GDFT_ERR_INVALID


def test_chunked_workspace_is_bounded_by_the_chunk(built_lib):
    """The chunked path's workspace depends on the chunk, not on the grid (host-only call)."""
    from graddft_gb300 import _lib

    lib = _lib.load(built_lib)
    small, big = ctypes.c_size_t(), ctypes.c_size_t()
    assert lib.gdft_chunked_workspace_bytes(512, 1 << 16, _lib.GDFT_TF32X3, None, ctypes.byref(small)) == 0
    assert lib.gdft_chunked_workspace_bytes(512, 1 << 17, _lib.GDFT_TF32X3, None, ctypes.byref(big)) == 0
    assert 1.9 < big.value / small.value < 2.1
    full = ctypes.c_size_t()
    mol = _lib.GdftMolecule()
    assert lib.gdft_molecule_bytes(1 << 20, 512, _lib.GDFT_TF32X3, ctypes.byref(full)) == 0
    assert small.value < full.value / 8  # 2^16-point chunks against the resident 2^20-point tables
    assert lib.gdft_chunked_workspace_bytes(512, 1000, _lib.GDFT_FP64, None, ctypes.byref(small)) == \
        _lib.GDFT_ERR_INVALID  # chunks are multiples of 256 points
