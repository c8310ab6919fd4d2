"""Batches of molecules of different sizes in one device call, capturable in a CUDA graph.

A training step over a dataset (train.py:34-218 applied to every molecule,
loss sum_m (E_m - E_ref_m)^2) becomes one ``gdft_neural_batch_xc`` call: each
molecule's density contraction, one network pass over all molecules' grid
points, the per-molecule energies and loss cotangents on the device, and each
molecule's V_xc contraction.  Nothing in the step synchronises the host, so
``capture()`` records it once as a CUDA graph and ``replay()`` re-runs it with
whatever the static input buffers (density matrices, parameters, reference
energies) hold.
"""
from __future__ import annotations

import ctypes
from typing import Optional, Sequence

import torch

from . import _lib, engine
from ._lib import GdftMolecule, check
from .functional import CLIP

F64 = torch.float64


class NeuralBatch:
    """Static buffers and workspace for a fixed set of molecules and one neural functional."""

    def __init__(self, molecules: Sequence, functional, clip_cte: float = CLIP):
        if not molecules:
            raise ValueError("a batch needs at least one molecule")
        self.residents = [m.resident() for m in molecules]
        self.device = self.residents[0].device
        self.net = functional.network(clip_cte)
        if self.net.precision != "tf32x3":
            raise NotImplementedError("batched steps run the TF32x3 network form (functional.precision='tf32x3')")
        n = len(molecules)
        self.n = n
        self.descs = (GdftMolecule * n)(*[r.desc for r in self.residents])
        self.rdm1 = [m._rdm1().clone() for m in molecules]
        self.ehf = [engine.as_device_f64(functional._ehf(m), self.device) for m in molecules]
        for r, e in zip(self.residents, self.ehf):
            if tuple(e.shape) != (2, 2, r.n_grid):
                raise ValueError(f"ehf must be (2, 2, {r.n_grid}), got {tuple(e.shape)}")
        self.vxc = [torch.empty((2, r.n_ao, r.n_ao), dtype=F64, device=self.device) for r in self.residents]
        self.energies = torch.empty(n, dtype=F64, device=self.device)
        self.loss = torch.empty((), dtype=F64, device=self.device)
        self.eref = torch.zeros(n, dtype=F64, device=self.device)
        self.params = torch.zeros(self.net.n_params, dtype=F64, device=self.device)
        self.dparams = torch.empty(self.net.n_params, dtype=F64, device=self.device)
        nbytes = ctypes.c_size_t()
        check(_lib.load().gdft_neural_batch_workspace_bytes(n, self.descs, ctypes.byref(self.net.desc),
                                                            ctypes.byref(nbytes)))
        self.ws = torch.zeros(nbytes.value, dtype=torch.uint8, device=self.device)  # error word 0
        ptrs = lambda ts: (ctypes.c_void_p * n)(*[t.data_ptr() for t in ts])  # noqa: E731
        self._h_rdm1, self._h_ehf, self._h_vxc = ptrs(self.rdm1), ptrs(self.ehf), ptrs(self.vxc)
        self.use_eref = False
        self.graph: Optional[torch.cuda.CUDAGraph] = None

    @property
    def n_points(self) -> int:
        return sum(r.n_grid for r in self.residents)

    def set_inputs(self, params=None, rdm1s=None, eref=None):
        """Copy new inputs into the static buffers (device copies, stream-ordered)."""
        if params is not None:
            self.params.copy_(params if isinstance(params, torch.Tensor) and params.ndim == 1
                              else self.net.flatten(params, self.device))
        if rdm1s is not None:
            for dst, src in zip(self.rdm1, rdm1s):
                dst.copy_(engine.as_device_f64(src, self.device))
        if eref is not None:
            self.eref.copy_(torch.as_tensor(eref, dtype=F64, device=self.device))
            self.use_eref = True

    def _launch(self):
        check(_lib.load().gdft_neural_batch_xc(
            self.n, self.descs, self._h_rdm1, self._h_ehf, ctypes.byref(self.net.desc), engine._ptr(self.params),
            engine._ptr(self.eref) if self.use_eref else None, engine._ptr(self.energies), engine._ptr(self.loss),
            self._h_vxc, engine._ptr(self.dparams), engine._ptr(self.ws), self.ws.numel(),
            engine._stream(self.device)))

    def step(self, params=None, rdm1s=None, eref=None):
        """(loss, energies (n,), [dloss/dD_m], dloss/dtheta flat) for the current inputs."""
        self.set_inputs(params, rdm1s, eref)
        self._launch()
        return self.loss, self.energies, self.vxc, self.dparams

    def capture(self):
        """Record one step as a CUDA graph (after one eager step has warmed the library up)."""
        self._launch()
        torch.cuda.synchronize(self.device)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self._launch()
        return self.graph

    def replay(self):
        if self.graph is None:
            raise RuntimeError("capture() first")
        self.graph.replay()
        return self.loss, self.energies, self.vxc, self.dparams

    def status(self) -> int:
        """Synchronise and raise if a kernel of the batch recorded an expired bounded wait (the batch
        workspace's persistent error word, where every molecule's stages and the network fold theirs)."""
        st = ctypes.c_int32()
        check(_lib.load().gdft_neural_batch_status(engine._ptr(self.ws), self.ws.numel(), ctypes.byref(st),
                                                   engine._stream(self.device)))
        return st.value
