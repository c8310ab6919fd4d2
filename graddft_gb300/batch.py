"""Batches of molecules of different sizes: in one device call, capturable in a CUDA graph
(``NeuralBatch``, resident AO tables), or side by side on several CUDA streams with the AO
tables recomputed per grid chunk (``ChunkedBatch``).

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


class ChunkedBatch:
    """Molecules whose AO tables are recomputed per grid chunk (``engine.ChunkedResident``), evaluated side
    by side on several CUDA streams.

    One molecule at a time leaves most SMs idle for the small ones (the chunk of a 24-AO molecule is a few
    dozen 128-point tiles per contraction).  The molecules are dealt longest first (cost n_grid * n_ao^2,
    the contractions' work) to the stream with the least cost queued so far; the molecules of one stream
    run one after another there and share that stream's workspace pool.  A step makes every stream wait
    for the caller's stream first and the caller's stream wait for all of them at the end, so it orders
    like any single-stream call.  Molecules whose chunk size is still "auto" are tuned on the caller's
    stream the first time (their timing must not overlap other work).
    """

    def __init__(self, residents: Sequence[engine.ChunkedResident], n_streams: int = 3):
        if not residents:
            raise ValueError("a batch needs at least one molecule")
        if n_streams < 1:
            raise ValueError(f"n_streams must be positive, got {n_streams}")
        self.residents = list(residents)
        self.device = self.residents[0].device
        n_streams = min(n_streams, len(self.residents))
        self.streams = [torch.cuda.Stream(self.device) for _ in range(n_streams)]
        self.pools = [{} for _ in range(n_streams)]
        self.assignment = schedule_longest_first([r.n_grid * r.n_ao ** 2 for r in self.residents], n_streams)
        for s, idxs in enumerate(self.assignment):
            for i in idxs:
                self.residents[i].use_workspace_pool(self.pools[s])

    def neural_xc_energy_and_grads(self, rdm1s, net: engine.Network, flat_params, ehfs, exc_out: torch.Tensor,
                                   vxc_outs=None, dparams_out: Optional[torch.Tensor] = None):
        """E_m into exc_out[m], V_xc of molecule m into vxc_outs[m] (or none), dE_m/dtheta into row m of
        dparams_out (or none), for every molecule, on the streams."""
        n = len(self.residents)
        if exc_out.shape != (n,):
            raise ValueError(f"exc_out must be ({n},), got {tuple(exc_out.shape)}")
        want_v, want_d = vxc_outs is not None, dparams_out is not None

        def call(i):
            self.residents[i].neural_xc_energy_and_grads(
                rdm1s[i], net, flat_params, ehfs[i], want_vxc=want_v, want_dparams=want_d, exc_out=exc_out[i],
                vxc_out=vxc_outs[i] if want_v else None, dparams_out=dparams_out[i] if want_d else None)

        done = set()
        for i, r in enumerate(self.residents):  # chunk sizes still to tune: alone, on the caller's stream
            if r.chunk == "auto":
                call(i)
                done.add(i)
        caller = torch.cuda.current_stream(self.device)
        for stream, idxs in zip(self.streams, self.assignment):
            stream.wait_stream(caller)
            with torch.cuda.stream(stream):
                for i in idxs:
                    if i not in done:
                        call(i)
        for stream in self.streams:
            caller.wait_stream(stream)
        return exc_out, vxc_outs, dparams_out

    def status(self) -> int:
        """Synchronise and raise if a kernel of any molecule recorded an expired bounded wait."""
        st = 0
        for r in self.residents:
            st = r.status() or st
        return st


def schedule_longest_first(costs: Sequence[float], n_streams: int) -> list:
    """Indices dealt to n_streams queues: longest first, each to the queue with the least cost so far (ties to
    the lowest queue), the order within a queue the dealing order."""
    queues = [[] for _ in range(n_streams)]
    load = [0.0] * n_streams
    for i in sorted(range(len(costs)), key=lambda j: (-costs[j], j)):
        q = min(range(n_streams), key=lambda k: (load[k], k))
        queues[q].append(i)
        load[q] += costs[i]
    return queues
