"""Failure detection and the DLPack boundary on the GPU.

A bounded device wait that runs out (a probe kernel waits on an mbarrier that
nothing arrives on) must reach the host as GDFT_ERR_DEVICE and the Python
layer as an exception, leave the context usable, and clear on read.  Inputs
handed over as DLPack producers (what a jax.Array is to this library) must go
through a full energy_predictor call.
"""
import ctypes

import numpy as np
import pytest
import torch

import oracle as O
from graddft_gb300 import synthetic

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib(built_lib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from graddft_gb300 import _lib

    return _lib


class DLPackOnly:
    """An array that offers nothing but the DLPack protocol (as a jax.Array does to torch)."""

    def __init__(self, t):
        self._t = t

    def __dlpack__(self, *args, **kwargs):
        return self._t.__dlpack__(*args, **kwargs)

    def __dlpack_device__(self):
        return self._t.__dlpack_device__()


def test_expired_wait_is_reported_and_cleared(lib):
    from graddft_gb300 import engine

    wl = synthetic.make_workload(256, 16, 3, seed=5, box_angstrom=6.0, centre_box_angstrom=4.0)
    ao, g1, g2 = O.eval_ao_planes(wl.basis, wl.coords)
    r = engine.Resident.from_tables(ao, g1, g2, wl.weights)
    assert r.status() == 0
    stream = engine._stream(r.device)
    L = lib.load()
    assert L.gdft_selftest_wait_expiry(ctypes.byref(r.desc), engine._ptr(r.ws), r.ws.numel(), 0, stream) \
        == lib.GDFT_ERR_INVALID
    lib.check(L.gdft_selftest_wait_expiry(ctypes.byref(r.desc), engine._ptr(r.ws), r.ws.numel(), 256, stream))
    st = ctypes.c_int32()
    rc = L.gdft_device_status(ctypes.byref(r.desc), engine._ptr(r.ws), r.ws.numel(), ctypes.byref(st), stream)
    assert rc == lib.GDFT_ERR_DEVICE and st.value == lib.GDFT_WAIT_EXPIRY_PROBE
    assert b"expired" in L.gdft_last_error()
    # read once, then clear; the Python layer raises for the next expiry
    assert r.status() == 0
    lib.check(L.gdft_selftest_wait_expiry(ctypes.byref(r.desc), engine._ptr(r.ws), r.ws.numel(), 256, stream))
    with pytest.raises(lib.GdftError, match="expired"):
        r.status()
    # the context is still usable: a full evaluation matches the oracle
    fn = engine.make_functional([lib.COL_LSDA, lib.COL_B88, lib.COL_LYP], [1.0])
    exc, vxc = r.xc_energy_and_grads(wl.rdm1, fn)
    e_ref, v_ref = O.xc_energy_and_grads("BLYP", wl.rdm1, ao, g1, g2, wl.weights)
    assert abs(float(exc) - e_ref) <= 1e-11 * abs(e_ref)
    assert np.max(np.abs(vxc.cpu().numpy() - v_ref)) <= 1e-11 * np.max(np.abs(v_ref))
    assert r.status() == 0


def test_dlpack_inputs_through_energy_predictor(lib, golden):
    import graddft_gb300 as G

    g = golden("compact")
    dl = lambda x: DLPackOnly(torch.as_tensor(np.asarray(x), dtype=torch.float64, device="cuda"))  # noqa: E731
    mol = G.Molecule(grid=G.Grid(coords=None, weights=dl(g["weights"])), atom_index=None, nuclear_pos=None,
                     ao=dl(g["ao"]), grad_ao=dl(g["grad_ao"]), grad_n_ao={2: dl(g["grad2_ao"])}, rdm1=dl(g["rdm1"]),
                     nuclear_repulsion=1.25, h1e=dl(g["h1e"]), vj=None, mo_coeff=None, mo_occ=None, mo_energy=None,
                     rep_tensor=dl(g["eri"]))
    E, F = G.energy_predictor(G.B88)({"params": {}}, mol)
    ref = float(g["predict_E_B88"])
    assert abs(float(E) - ref) <= 1e-11 * abs(ref)
    Fr = g["predict_F_B88"]
    assert np.max(np.abs(F.cpu().numpy() - Fr)) <= 1e-11 * np.max(np.abs(Fr))
