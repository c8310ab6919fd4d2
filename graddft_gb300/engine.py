"""Device-side engine: resident molecules, workspaces and calls into libgdft_xc.so.

PyTorch is used only for device memory and the current CUDA stream; all
arithmetic of the XC path runs in the library's kernels.
"""
from __future__ import annotations

import ctypes
from typing import Optional, Sequence

import torch

from . import _lib
from ._lib import GdftFunctional, GdftMolecule, GdftNetwork, check

F64 = torch.float64
PRECISIONS = {"fp64": _lib.GDFT_FP64, "tf32x3": _lib.GDFT_TF32X3}


def _ptr(t: Optional[torch.Tensor]):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _stream(device: torch.device) -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def as_device_f64(x, device) -> torch.Tensor:
    """Accept torch tensors, numpy arrays or any DLPack producer (e.g. jax.Array)."""
    if x is None:
        return None
    if not isinstance(x, torch.Tensor):
        if hasattr(x, "__dlpack__") and not hasattr(x, "__array_interface__"):
            x = torch.from_dlpack(x)
        else:
            x = torch.as_tensor(x)
    return x.to(device=device, dtype=F64).contiguous()


def require_cuda(device=None) -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("the GB300 XC path needs a CUDA device (there is no CPU fallback)")
    d = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    if d.type != "cuda":
        raise RuntimeError(f"device {d} is not a CUDA device (there is no CPU fallback)")
    return d


class Resident:
    """A molecule's grid and AO tables resident in HBM in the library's layout."""

    def __init__(self, n_grid: int, n_ao: int, precision: str = "fp64", device=None):
        lib = _lib.load()
        self.device = require_cuda(device)
        self.n_grid, self.n_ao = int(n_grid), int(n_ao)
        self.precision = precision
        prec = PRECISIONS[precision]
        nbytes = ctypes.c_size_t()
        check(lib.gdft_molecule_bytes(self.n_grid, self.n_ao, prec, ctypes.byref(nbytes)))
        self.buffer = torch.empty(nbytes.value, dtype=torch.uint8, device=self.device)
        self.desc = GdftMolecule()
        check(lib.gdft_molecule_init(ctypes.byref(self.desc), self.n_grid, self.n_ao, prec,
                                     _ptr(self.buffer), nbytes.value))
        wbytes = ctypes.c_size_t()
        check(lib.gdft_workspace_bytes(ctypes.byref(self.desc), ctypes.byref(wbytes)))
        self.ws = torch.zeros(wbytes.value, dtype=torch.uint8, device=self.device)  # error word starts at 0

    @property
    def nbytes(self) -> int:
        return self.buffer.numel() + self.ws.numel()

    @classmethod
    def from_tables(cls, ao, grad_ao, grad2_ao, weights, precision="fp64", device=None) -> "Resident":
        dev = require_cuda(device)
        ao = as_device_f64(ao, dev)
        r = cls(ao.shape[0], ao.shape[1], precision, dev)
        r.load(ao, grad_ao, grad2_ao, weights)
        return r

    def load(self, ao, grad_ao, grad2_ao, weights):
        ao = as_device_f64(ao, self.device)
        grad_ao = as_device_f64(grad_ao, self.device)
        grad2_ao = as_device_f64(grad2_ao, self.device)
        weights = as_device_f64(weights, self.device)
        if ao.shape != (self.n_grid, self.n_ao) or grad_ao.shape != (self.n_grid, self.n_ao, 3):
            raise ValueError(f"ao {tuple(ao.shape)} / grad_ao {tuple(grad_ao.shape)} do not match "
                             f"({self.n_grid}, {self.n_ao}[, 3])")
        if grad2_ao is not None and grad2_ao.shape != (self.n_grid, self.n_ao, 3):
            raise ValueError(f"grad_n_ao[2] {tuple(grad2_ao.shape)} does not match ({self.n_grid}, {self.n_ao}, 3)")
        if weights.shape != (self.n_grid,):
            raise ValueError(f"weights {tuple(weights.shape)} do not match ({self.n_grid},)")
        check(_lib.load().gdft_molecule_load(ctypes.byref(self.desc), _ptr(ao), _ptr(grad_ao), _ptr(grad2_ao),
                                             _ptr(weights), _stream(self.device)))

    @classmethod
    def from_basis(cls, basis_rows, coords, weights, precision="fp64", device=None) -> "Resident":
        """Evaluate a seeded Gaussian basis on the device (see graddft_gb300.synthetic)."""
        dev = require_cuda(device)
        basis_rows = as_device_f64(basis_rows, dev)
        coords = as_device_f64(coords, dev)
        weights = as_device_f64(weights, dev)
        r = cls(coords.shape[0], basis_rows.shape[0], precision, dev)
        check(_lib.load().gdft_molecule_eval_basis(ctypes.byref(r.desc), _ptr(basis_rows), _ptr(coords),
                                                   _ptr(weights), _stream(dev)))
        torch.cuda.current_stream(dev).synchronize()
        return r

    @classmethod
    def from_shells(cls, basis, coords, weights, precision="fp64", device=None) -> "Resident":
        """Evaluate a contracted Gaussian basis (``graddft_gb300.basis.ShellBasis``) straight into the
        resident tables: no (grid, ao) reference-layout arrays are formed."""
        dev = require_cuda(device)
        coords = as_device_f64(coords, dev)
        weights = as_device_f64(weights, dev)
        if coords.ndim != 2 or coords.shape[1] != 3 or weights.shape != (coords.shape[0],):
            raise ValueError(f"coords {tuple(coords.shape)} / weights {tuple(weights.shape)} must be (grid, 3) / (grid,)")
        desc, _keep = basis.device_desc(dev)
        r = cls(coords.shape[0], desc.n_ao, precision, dev)
        check(_lib.load().gdft_molecule_eval_shells(ctypes.byref(r.desc), ctypes.byref(desc), _ptr(coords),
                                                    _ptr(weights), _stream(dev)))
        torch.cuda.current_stream(dev).synchronize()
        return r

    def ao_planes(self) -> torch.Tensor:
        """The FP64 form's resident tables as a (5, n_grid_pad, ld) view: phi, d_x, d_y, d_z, lap phi."""
        if self.precision != "fp64":
            raise ValueError("the resident tables are FP64 planes only in the FP64 form")
        np_, ld = int(self.desc.n_grid_pad), int(self.desc.ld)
        off = (np_ * 8 + 255) // 256 * 256  # after the weights
        return self.buffer[off:off + 5 * np_ * ld * 8].view(torch.float64).view(5, np_, ld)

    # ------------------------------------------------------------------ calls
    def density(self, rdm1, want=("rho", "grad_rho", "lapl", "tau")):
        rdm1 = self._rdm1(rdm1)
        n = self.n_grid
        out = {
            "rho": torch.empty((n, 2), dtype=F64, device=self.device) if "rho" in want else None,
            "grad_rho": torch.empty((n, 2, 3), dtype=F64, device=self.device) if "grad_rho" in want else None,
            "lapl": torch.empty((n, 2), dtype=F64, device=self.device) if "lapl" in want else None,
            "tau": torch.empty((n, 2), dtype=F64, device=self.device) if "tau" in want else None,
        }
        check(_lib.load().gdft_density(ctypes.byref(self.desc), _ptr(rdm1), _ptr(out["rho"]), _ptr(out["grad_rho"]),
                                       _ptr(out["lapl"]), _ptr(out["tau"]), _ptr(self.ws), self.ws.numel(),
                                       _stream(self.device)))
        return out

    def xc_energy_and_grads(self, rdm1, fn: GdftFunctional, ehf=None, want_vxc=True, exc_out=None, vxc_out=None):
        rdm1 = self._rdm1(rdm1)
        ehf_t = as_device_f64(ehf, self.device)
        n_omega = 0
        if ehf_t is not None:
            if ehf_t.ndim != 3 or ehf_t.shape[1] != 2 or ehf_t.shape[2] != self.n_grid:
                raise ValueError(f"ehf must be (omega, 2, {self.n_grid}), got {tuple(ehf_t.shape)}")
            n_omega = ehf_t.shape[0]
        exc = exc_out if exc_out is not None else torch.empty((), dtype=F64, device=self.device)
        vxc = None
        if want_vxc:
            vxc = vxc_out if vxc_out is not None else torch.empty((2, self.n_ao, self.n_ao), dtype=F64,
                                                                   device=self.device)
        check(_lib.load().gdft_xc_energy_and_grads(ctypes.byref(self.desc), _ptr(rdm1), ctypes.byref(fn),
                                                   _ptr(ehf_t), n_omega, _ptr(exc), _ptr(vxc), _ptr(self.ws),
                                                   self.ws.numel(), _stream(self.device)))
        return exc, vxc

    def xc_energy_grads_hf(self, rdm1, fn: GdftFunctional, ehf, want_vxc=True):
        """(E_xc, V_xc, g): g (grid,) = dE_xc/d ehf[w][s][r] of the functional's HF column (the sum of ehf)."""
        rdm1 = self._rdm1(rdm1)
        ehf_t = as_device_f64(ehf, self.device)
        if ehf_t is None or ehf_t.ndim != 3 or ehf_t.shape[1] != 2 or ehf_t.shape[2] != self.n_grid:
            raise ValueError(f"ehf must be (omega, 2, {self.n_grid})")
        exc = torch.empty((), dtype=F64, device=self.device)
        vxc = torch.empty((2, self.n_ao, self.n_ao), dtype=F64, device=self.device) if want_vxc else None
        ghf = torch.empty(self.n_grid, dtype=F64, device=self.device)
        check(_lib.load().gdft_xc_energy_grads_hf(ctypes.byref(self.desc), _ptr(rdm1), ctypes.byref(fn), _ptr(ehf_t),
                                                  ehf_t.shape[0], _ptr(exc), _ptr(vxc), _ptr(ghf), _ptr(self.ws),
                                                  self.ws.numel(), _stream(self.device)))
        return exc, vxc, ghf

    def vxc_from_potentials(self, pot, vxc_out=None):
        """V_s = sum_r [c0 phi phi + sum_j c_j phi d_j phi + c4 phi lap phi + c5 sum_j d_j phi d_j phi], pot (2, 6, grid)."""
        pot = as_device_f64(pot, self.device)
        if pot.shape != (2, 6, self.n_grid):
            raise ValueError(f"potentials must be (2, 6, {self.n_grid}), got {tuple(pot.shape)}")
        vxc = vxc_out if vxc_out is not None else torch.empty((2, self.n_ao, self.n_ao), dtype=F64, device=self.device)
        check(_lib.load().gdft_vxc_from_potentials(ctypes.byref(self.desc), _ptr(pot), _ptr(vxc), _ptr(self.ws),
                                                   self.ws.numel(), _stream(self.device)))
        return vxc

    def neural_xc_energy_and_grads(self, rdm1, net: "Network", flat_params, ehf, want_vxc=True,
                                   want_dparams=False, exc_out=None, vxc_out=None, dparams_out=None):
        """E_xc, V_xc = dE/dD and dE/dtheta of a DM21-style neural functional (flat FP64 parameters)."""
        rdm1 = self._rdm1(rdm1)
        ehf_t = as_device_f64(ehf, self.device)
        if ehf_t is None or ehf_t.shape != (2, 2, self.n_grid):
            raise ValueError(f"ehf must be (2, 2, {self.n_grid}) for the DM21 inputs, got "
                             f"{None if ehf_t is None else tuple(ehf_t.shape)}")
        flat = as_device_f64(flat_params, self.device)
        if flat.ndim != 1 or flat.numel() != net.n_params:
            raise ValueError(f"flat parameters must hold {net.n_params} values, got {tuple(flat.shape)}")
        ws = self._neural_ws(net)
        exc = exc_out if exc_out is not None else torch.empty((), dtype=F64, device=self.device)
        vxc = None
        if want_vxc:
            vxc = vxc_out if vxc_out is not None else torch.empty((2, self.n_ao, self.n_ao), dtype=F64,
                                                                   device=self.device)
        dp = None
        if want_dparams:
            dp = dparams_out if dparams_out is not None else torch.empty(net.n_params, dtype=F64, device=self.device)
        check(_lib.load().gdft_neural_xc_energy_and_grads(
            ctypes.byref(self.desc), _ptr(rdm1), ctypes.byref(net.desc), _ptr(flat), _ptr(ehf_t), _ptr(exc),
            _ptr(vxc), _ptr(dp), _ptr(ws), ws.numel(), _stream(self.device)))
        return exc, vxc, dp

    def neural_xc_hf_grads(self, rdm1, net: "Network", flat_params, ehf, want_vxc=False):
        """(E_xc, V_xc or None, g_dens, g_cin) in one network pass: g = dE_xc/d ehf (2, 2, grid) through the
        HF densities and through the HF inputs."""
        rdm1 = self._rdm1(rdm1)
        ehf_t = as_device_f64(ehf, self.device)
        if ehf_t is None or ehf_t.shape != (2, 2, self.n_grid):
            raise ValueError(f"ehf must be (2, 2, {self.n_grid})")
        flat = as_device_f64(flat_params, self.device)
        ws = self._neural_ws(net)
        exc = torch.empty((), dtype=F64, device=self.device)
        g_dens = torch.empty((2, 2, self.n_grid), dtype=F64, device=self.device)
        g_cin = torch.empty((2, 2, self.n_grid), dtype=F64, device=self.device)
        vxc = torch.empty((2, self.n_ao, self.n_ao), dtype=F64, device=self.device) if want_vxc else None
        check(_lib.load().gdft_neural_xc_hf_grads(ctypes.byref(self.desc), _ptr(rdm1), ctypes.byref(net.desc),
                                                  _ptr(flat), _ptr(ehf_t.contiguous()), _ptr(exc), _ptr(vxc),
                                                  _ptr(g_dens), _ptr(g_cin), _ptr(ws), ws.numel(),
                                                  _stream(self.device)))
        return exc, vxc, g_dens, g_cin

    def neural_xc_hvp(self, rdm1, net: "Network", flat_params, ehf, tangent, want_value=False, want_drdm1=True,
                      want_dparams=True):
        """Gradients of L = <tangent, V_xc(D, theta)>: (L, dL/dD, dL/dtheta) (second-order adjoint)."""
        rdm1 = self._rdm1(rdm1)
        g = self._rdm1(tangent)
        ehf_t = as_device_f64(ehf, self.device)
        if ehf_t is None or ehf_t.shape != (2, 2, self.n_grid):
            raise ValueError(f"ehf must be (2, 2, {self.n_grid})")
        flat = as_device_f64(flat_params, self.device)
        if flat.ndim != 1 or flat.numel() != net.n_params:
            raise ValueError(f"flat parameters must hold {net.n_params} values, got {tuple(flat.shape)}")
        ws = self._hvp_ws(net)
        val = torch.empty((), dtype=F64, device=self.device) if want_value else None
        hd = torch.empty((2, self.n_ao, self.n_ao), dtype=F64, device=self.device) if want_drdm1 else None
        hp = torch.empty(net.n_params, dtype=F64, device=self.device) if want_dparams else None
        check(_lib.load().gdft_neural_xc_hvp(ctypes.byref(self.desc), _ptr(rdm1), ctypes.byref(net.desc), _ptr(flat),
                                             _ptr(ehf_t), _ptr(g), _ptr(val), _ptr(hd), _ptr(hp), _ptr(ws),
                                             ws.numel(), _stream(self.device)))
        return val, hd, hp

    # Workspaces of the network passes, one per network shape and form: callers that mix networks (the
    # DM21 inputs of the default network beside a functional's own, say) would otherwise reallocate and
    # zero a workspace of gigabytes on every switch.  The cache drops its least recently used entry.
    _WS_KEEP = 4

    def _cached_ws(self, name: str, net: "Network", size_fn) -> torch.Tensor:
        cache = self.__dict__.setdefault(name, {})
        ws = cache.pop(net.key, None)  # re-inserted last: the dict's order is least recently used first
        if ws is None:
            nbytes = ctypes.c_size_t()
            check(size_fn(ctypes.byref(self.desc), ctypes.byref(net.desc), ctypes.byref(nbytes)))
            if len(cache) >= self._WS_KEEP:
                self._retire_ws(cache.pop(next(iter(cache))))
            ws = torch.zeros(nbytes.value, dtype=torch.uint8, device=self.device)  # error word 0
        cache[net.key] = ws
        return ws

    def _retire_ws(self, ws: torch.Tensor) -> None:
        """Read a dropped workspace's error word before it goes: an expired bounded wait recorded there
        is kept and reported by the next status()."""
        st = ctypes.c_int32()
        rc = _lib.load().gdft_device_status(ctypes.byref(self.desc), _ptr(ws), ws.numel(), ctypes.byref(st),
                                            _stream(self.device))
        if rc == _lib.GDFT_ERR_DEVICE:
            self.__dict__["_sticky_status"] = st.value
        else:
            check(rc)

    def _hvp_ws(self, net: "Network") -> torch.Tensor:
        return self._cached_ws("_hws", net, _lib.load().gdft_neural_hvp_workspace_bytes)

    def _neural_ws(self, net: "Network") -> torch.Tensor:
        return self._cached_ws("_nws", net, _lib.load().gdft_neural_workspace_bytes)

    def status(self) -> int:
        """Synchronise and raise if a kernel recorded an expired bounded wait since the last query
        (including one recorded in a network workspace the cache has since dropped)."""
        st = ctypes.c_int32()
        check(_lib.load().gdft_device_status(ctypes.byref(self.desc), _ptr(self.ws), self.ws.numel(),
                                             ctypes.byref(st), _stream(self.device)))
        for name in ("_nws", "_hws"):
            for ws in self.__dict__.get(name, {}).values():
                check(_lib.load().gdft_device_status(ctypes.byref(self.desc), _ptr(ws), ws.numel(),
                                                     ctypes.byref(st), _stream(self.device)))
        sticky = self.__dict__.pop("_sticky_status", 0)
        if sticky:
            raise _lib.GdftError(f"a device-side wait expired (code {sticky}) in a network workspace since "
                                 "dropped from the cache; results of the calls before it are invalid")
        return st.value

    def _rdm1(self, rdm1) -> torch.Tensor:
        rdm1 = as_device_f64(rdm1, self.device)
        if rdm1.shape != (2, self.n_ao, self.n_ao):
            raise ValueError(f"rdm1 must be (2, {self.n_ao}, {self.n_ao}), got {tuple(rdm1.shape)}")
        return rdm1


class ChunkedResident:
    """A molecule whose AO tables are never held for the whole grid.

    The grid is processed in chunks of ``chunk`` points; each chunk's AO tables
    are evaluated from the basis into a chunk buffer and contracted at once
    (gdft_xc_energy_and_grads_chunked): phi is recomputed per chunk instead of
    stored, so the device memory is the basis, the grid and one chunk's tables
    and workspace (a few GB where the resident tables of 2^20 points x 512 AOs
    take 64 GiB plus the 48 GiB V_xc operand).  The same calls as ``Resident``
    for the functional and network passes.
    """

    def __init__(self, basis, coords, weights, precision: str = "fp64", chunk=1 << 16, device=None,
                 workspace_pool: Optional[dict] = None):
        """``chunk``: grid points per chunk (a multiple of 256), or "auto" to let ``autotune`` pick it on
        the first call (timed once per problem bucket and cached on disk).  ``workspace_pool``: a dict
        shared by several molecules evaluated one after another, so that they reuse one workspace per
        network shape (grown to the largest molecule) instead of holding one each."""
        self.device = require_cuda(device)
        if precision not in PRECISIONS:
            raise ValueError(f"precision must be one of {sorted(PRECISIONS)}, got {precision!r}")
        if chunk != "auto" and (int(chunk) < 256 or int(chunk) % 256):
            raise ValueError(f"chunk must be a positive multiple of 256 grid points or 'auto', got {chunk}")
        self.precision, self.chunk = precision, (chunk if chunk == "auto" else int(chunk))
        self.coords = as_device_f64(coords, self.device)
        self.weights = as_device_f64(weights, self.device)
        if self.coords.ndim != 2 or self.coords.shape[1] != 3 or self.weights.shape != (self.coords.shape[0],):
            raise ValueError(f"coords {tuple(self.coords.shape)} / weights {tuple(self.weights.shape)} must be "
                             "(grid, 3) / (grid,)")
        self.n_grid = int(self.coords.shape[0])
        if hasattr(basis, "device_desc"):  # a contracted ShellBasis
            self._desc, self._keep = basis.device_desc(self.device)
            self._rows = None
            self.n_ao = int(self._desc.n_ao)
        else:  # the synthetic rows of gdft_molecule_eval_basis, (n_ao, 8)
            self._desc, self._keep = None, None
            self._rows = as_device_f64(basis, self.device)
            if self._rows.ndim != 2 or self._rows.shape[1] != 8:
                raise ValueError(f"basis rows must be (n_ao, 8), got {tuple(self._rows.shape)}")
            self.n_ao = int(self._rows.shape[0])
        self._ws = workspace_pool if workspace_pool is not None else {}

    def _basis_args(self):
        return (None if self._desc is None else ctypes.byref(self._desc)), _ptr(self._rows)

    def use_workspace_pool(self, pool: dict) -> None:
        """Take workspaces from ``pool`` from now on (molecules that share a pool must run one after another
        on one stream; ``batch.ChunkedBatch`` gives each of its streams its own)."""
        self._ws = pool

    def workspace_bytes(self, chunk: int, net: Optional["Network"] = None) -> int:
        nbytes = ctypes.c_size_t()
        check(_lib.load().gdft_chunked_workspace_bytes(self.n_ao, int(chunk), PRECISIONS[self.precision],
                                                       None if net is None else ctypes.byref(net.desc),
                                                       ctypes.byref(nbytes)))
        return nbytes.value

    def workspace(self, net: Optional["Network"] = None) -> torch.Tensor:
        key = None if net is None else net.key
        need = self.workspace_bytes(self.chunk, net)
        ws = self._ws.get(key)
        if ws is None or ws.numel() < need:
            if ws is not None:  # report what the smaller workspace recorded before it goes
                st = ctypes.c_int32()
                check(_lib.load().gdft_chunked_status(_ptr(ws), ws.numel(), ctypes.byref(st), _stream(self.device)))
            self._ws.pop(key, None)
            ws = self._ws[key] = torch.zeros(need, dtype=torch.uint8, device=self.device)  # error word 0
        return ws

    def _resolve_chunk(self, net: Optional["Network"], call) -> None:
        """Pick the chunk size with the autotuner when it was left to "auto" (the first call times the
        candidates with the caller's own arguments)."""
        if self.chunk != "auto":
            return
        from . import autotune

        key = autotune.bucket_key(self.n_ao, self.precision, None if net is None else net.key, self.device)

        def run(c):
            self.chunk = c
            call()

        self.chunk = autotune.choose(key, run, lambda c: self.workspace_bytes(c, net), self.n_grid, self.device)
        self._ws.pop(None if net is None else net.key, None)  # the timing may have grown it past the chosen size

    @property
    def nbytes(self) -> int:
        return sum(ws.numel() for ws in self._ws.values())

    def _rdm1(self, rdm1) -> torch.Tensor:
        rdm1 = as_device_f64(rdm1, self.device)
        if rdm1.shape != (2, self.n_ao, self.n_ao):
            raise ValueError(f"rdm1 must be (2, {self.n_ao}, {self.n_ao}), got {tuple(rdm1.shape)}")
        return rdm1

    def xc_energy_and_grads(self, rdm1, fn: GdftFunctional, ehf=None, want_vxc=True, exc_out=None, vxc_out=None):
        rdm1 = self._rdm1(rdm1)
        ehf_t = as_device_f64(ehf, self.device)
        n_omega = 0
        if ehf_t is not None:
            if ehf_t.ndim != 3 or ehf_t.shape[1] != 2 or ehf_t.shape[2] != self.n_grid:
                raise ValueError(f"ehf must be (omega, 2, {self.n_grid}), got {tuple(ehf_t.shape)}")
            n_omega = ehf_t.shape[0]
        exc = exc_out if exc_out is not None else torch.empty((), dtype=F64, device=self.device)
        vxc = None
        if want_vxc:
            vxc = vxc_out if vxc_out is not None else torch.empty((2, self.n_ao, self.n_ao), dtype=F64,
                                                                   device=self.device)
        self._resolve_chunk(None, lambda: self.xc_energy_and_grads(rdm1, fn, ehf, want_vxc, exc, vxc))
        ws = self.workspace()
        shells, rows = self._basis_args()
        check(_lib.load().gdft_xc_energy_and_grads_chunked(
            shells, rows, self.n_ao, _ptr(self.coords), _ptr(self.weights), self.n_grid, self.chunk,
            PRECISIONS[self.precision], _ptr(rdm1), ctypes.byref(fn), _ptr(ehf_t), n_omega, _ptr(exc), _ptr(vxc),
            _ptr(ws), ws.numel(), _stream(self.device)))
        return exc, vxc

    def neural_xc_energy_and_grads(self, rdm1, net: "Network", flat_params, ehf, want_vxc=True,
                                   want_dparams=False, exc_out=None, vxc_out=None, dparams_out=None):
        rdm1 = self._rdm1(rdm1)
        ehf_t = as_device_f64(ehf, self.device)
        if ehf_t is None or ehf_t.shape != (2, 2, self.n_grid):
            raise ValueError(f"ehf must be (2, 2, {self.n_grid}) for the DM21 inputs")
        flat = as_device_f64(flat_params, self.device)
        if flat.ndim != 1 or flat.numel() != net.n_params:
            raise ValueError(f"flat parameters must hold {net.n_params} values, got {tuple(flat.shape)}")
        exc = exc_out if exc_out is not None else torch.empty((), dtype=F64, device=self.device)
        vxc = (vxc_out if vxc_out is not None else torch.empty((2, self.n_ao, self.n_ao), dtype=F64,
                                                               device=self.device)) if want_vxc else None
        dp = (dparams_out if dparams_out is not None else torch.empty(net.n_params, dtype=F64, device=self.device)
              ) if want_dparams else None
        self._resolve_chunk(net, lambda: self.neural_xc_energy_and_grads(rdm1, net, flat, ehf_t, want_vxc,
                                                                         want_dparams, exc, vxc, dp))
        ws = self.workspace(net)
        shells, rows = self._basis_args()
        check(_lib.load().gdft_neural_xc_energy_and_grads_chunked(
            shells, rows, self.n_ao, _ptr(self.coords), _ptr(self.weights), self.n_grid, self.chunk,
            PRECISIONS[self.precision], _ptr(rdm1), ctypes.byref(net.desc), _ptr(flat), _ptr(ehf_t.contiguous()),
            _ptr(exc), _ptr(vxc), _ptr(dp), _ptr(ws), ws.numel(), _stream(self.device)))
        return exc, vxc, dp

    def status(self) -> int:
        """Synchronise and raise if a kernel recorded an expired bounded wait since the last query."""
        st = ctypes.c_int32()
        for ws in self._ws.values():
            check(_lib.load().gdft_chunked_status(_ptr(ws), ws.numel(), ctypes.byref(st), _stream(self.device)))
        return st.value

    def __getattr__(self, name):
        if name in ("density", "vxc_from_potentials", "neural_xc_hf_grads", "neural_xc_hvp", "xc_energy_grads_hf"):
            raise NotImplementedError(f"{name} needs the AO tables of the whole grid; build the molecule with "
                                      "resident tables (molecule_from_basis without recompute_chunk)")
        raise AttributeError(name)


class Network:
    """Shape and constants of a DM21-style coefficient network, and its flat parameter layout.

    The flat order (the one include/gdft.h documents) follows the flax module
    names of DM21.default_nn (functional.py:797-822, names at :876-891):
    Dense_0 kernel/bias, then per layer Dense_i kernel/bias and LayerNorm_{i-1}
    scale/bias, then the head Dense_{L+1} kernel/bias.
    """

    def __init__(self, n_layers: int = 6, width: int = 256, n_in: int = 11, n_out: int = 3,
                 squash_offset: float = 1e-4, sigmoid_scale: float = 2.0, ln_eps: float = 1e-6,
                 clip: float = 1e-30, precision: str = "fp64"):
        self.desc = GdftNetwork()
        d = self.desc
        d.n_in, d.width, d.n_layers, d.n_out = int(n_in), int(width), int(n_layers), int(n_out)
        if precision not in PRECISIONS:
            raise ValueError(f"network precision must be one of {sorted(PRECISIONS)}, got {precision!r}")
        d.precision = PRECISIONS[precision]
        self.precision = precision
        d.squash_offset, d.sigmoid_scale, d.ln_eps, d.clip = (float(squash_offset), float(sigmoid_scale),
                                                              float(ln_eps), float(clip))
        self.n_layers, self.width, self.n_in, self.n_out = d.n_layers, d.width, d.n_in, d.n_out
        self.key = (d.n_in, d.width, d.n_layers, d.n_out, d.precision)
        self.entries = self._entries()
        self.n_params = sum(int(torch.Size(shape).numel()) for _, _, shape in self.entries)

    def _entries(self):
        W, L = self.width, self.n_layers
        ent = [("Dense_0", "kernel", (self.n_in, W)), ("Dense_0", "bias", (W,))]
        for i in range(1, L + 1):
            ent += [(f"Dense_{i}", "kernel", (W, W)), (f"Dense_{i}", "bias", (W,)),
                    (f"LayerNorm_{i - 1}", "scale", (W,)), (f"LayerNorm_{i - 1}", "bias", (W,))]
        ent += [(f"Dense_{L + 1}", "kernel", (W, self.n_out)), (f"Dense_{L + 1}", "bias", (self.n_out,))]
        return ent

    def flatten(self, params, device) -> torch.Tensor:
        """flax-style {'params': {module: {leaf: array}}} -> one contiguous FP64 device vector."""
        p = params["params"] if "params" in params else params
        parts = []
        for mod, leaf, shape in self.entries:
            if mod not in p or leaf not in p[mod]:
                raise ValueError(f"params has no {mod}/{leaf}")
            t = as_device_f64(p[mod][leaf], device)
            if tuple(t.shape) != shape:
                raise ValueError(f"params {mod}/{leaf} has shape {tuple(t.shape)}, expected {shape}")
            parts.append(t.reshape(-1))
        return torch.cat(parts)

    def unflatten(self, flat: torch.Tensor):
        """The inverse of flatten: a flax-style nested dict of views into flat."""
        out, off = {}, 0
        for mod, leaf, shape in self.entries:
            n = int(torch.Size(shape).numel())
            out.setdefault(mod, {})[leaf] = flat[off:off + n].view(shape)
            off += n
        return {"params": out}


def selftest_umma() -> float:
    """Run the tensor-core self-test; returns the max abs error (0 when the device path is right)."""
    err = ctypes.c_double()
    check(_lib.load().gdft_selftest_umma(ctypes.byref(err)))
    return err.value


def make_functional(cols: Sequence[int], coeffs: Sequence[float], clip: float = 1e-30) -> GdftFunctional:
    cols, coeffs = list(cols), [float(c) for c in coeffs]
    if not 1 <= len(cols) <= _lib.MAX_COLS:
        raise ValueError(f"a functional needs 1..{_lib.MAX_COLS} energy-density columns, got {len(cols)}")
    if len(coeffs) not in (1, len(cols)):
        raise ValueError(f"{len(coeffs)} coefficients for {len(cols)} energy-density columns")
    fn = GdftFunctional()
    fn.n_cols = len(cols)
    for i, c in enumerate(cols):
        fn.cols[i] = int(c)
    fn.n_coeffs = len(coeffs)
    for i, c in enumerate(coeffs):
        fn.coeffs[i] = c
    fn.clip = float(clip)
    return fn


def fock(h1e, vj, vxc, clip=1e-30) -> torch.Tensor:
    dev = vxc.device
    n = vxc.shape[-1]
    h1e = as_device_f64(h1e, dev)
    vj = as_device_f64(vj, dev)
    out = torch.empty_like(vxc)
    check(_lib.load().gdft_fock(n, _ptr(h1e), _ptr(vj), _ptr(vxc.contiguous()), float(clip), _ptr(out),
                                _stream(dev)))
    return out


def _hf_form(form) -> int:
    if form not in PRECISIONS:
        raise ValueError(f"unknown form {form!r}; expected one of {sorted(PRECISIONS)}")
    return PRECISIONS[form]


def _hf_ws(n_grid: int, n_ao: int, n_omega: int, form: int, device) -> torch.Tensor:
    nbytes = ctypes.c_size_t()
    check(_lib.load().gdft_hf_workspace_bytes_form(n_grid, n_ao, n_omega, form, ctypes.byref(nbytes)))
    return torch.empty(nbytes.value, dtype=torch.uint8, device=device)


def _hf_status(ws: torch.Tensor, form: int) -> None:
    """The bounded-wait error word of a mixed-form exchange call (synchronises the stream)."""
    if form == _lib.GDFT_TF32X3:
        status = ctypes.c_int32()
        check(_lib.load().gdft_hf_device_status(_ptr(ws), ws.numel(), ctypes.byref(status), _stream(ws.device)))


def _chi(chi, ao):
    chi = as_device_f64(chi, ao.device)
    if chi.ndim != 4 or chi.shape[0] != ao.shape[0] or chi.shape[2] != 2 or chi.shape[3] != ao.shape[1]:
        raise ValueError(f"chi must be (grid, omega, 2, orbitals) = ({ao.shape[0]}, omega, 2, {ao.shape[1]}), "
                         f"got {tuple(chi.shape)}")
    return chi.contiguous()


def hf_energy_density(ao, rdm1, chi, form: str = "fp64") -> torch.Tensor:
    """molecule.py:507-541: ehf (omega, 2, grid) = -1/2 einsum("rwsc,sac,ra->wsr", chi, rdm1, ao).

    ``form`` "fp64" contracts on the FP64 GEMM, "tf32x3" on the block-scaled three-slice tensor-core GEMM.
    """
    dev = require_cuda(ao.device if isinstance(ao, torch.Tensor) and ao.is_cuda else None)
    code = _hf_form(form)
    ao = as_device_f64(ao, dev).contiguous()
    rdm1 = as_device_f64(rdm1, dev).contiguous()
    chi = _chi(chi, ao)
    n_grid, n_ao = ao.shape
    n_omega = chi.shape[1]
    out = torch.empty((n_omega, 2, n_grid), dtype=F64, device=dev)
    ws = _hf_ws(n_grid, n_ao, n_omega, code, dev)
    check(_lib.load().gdft_hf_energy_density_form(_ptr(ao), _ptr(rdm1), _ptr(chi), n_grid, n_ao, n_omega, code,
                                                  _ptr(out), _ptr(ws), ws.numel(), _stream(dev)))
    _hf_status(ws, code)
    return out


def hf_fock(ao, chi, g, form: str = "fp64") -> torch.Tensor:
    """sum over omega of molecule.py:545-685: F_s = -1/2 sum_w einsum("rw s b, w s r, r a -> s a b")."""
    dev = require_cuda(ao.device if isinstance(ao, torch.Tensor) and ao.is_cuda else None)
    code = _hf_form(form)
    ao = as_device_f64(ao, dev).contiguous()
    chi = _chi(chi, ao)
    n_grid, n_ao = ao.shape
    n_omega = chi.shape[1]
    g = as_device_f64(g, dev)
    if tuple(g.shape) != (n_omega, 2, n_grid):
        raise ValueError(f"g must be (omega, 2, grid) = ({n_omega}, 2, {n_grid}), got {tuple(g.shape)}")
    g = g.contiguous()
    out = torch.empty((2, n_ao, n_ao), dtype=F64, device=dev)
    ws = _hf_ws(n_grid, n_ao, n_omega, code, dev)
    check(_lib.load().gdft_hf_fock_form(_ptr(ao), _ptr(chi), _ptr(g), n_grid, n_ao, n_omega, code, _ptr(out),
                                        _ptr(ws), ws.numel(), _stream(dev)))
    _hf_status(ws, code)
    return out


def fock_add_hf(fock_, fock_hf, clip=1e-30) -> torch.Tensor:
    """train.py:200-210: fock = abs_clip(fock + F + F^T) (in place on a copy)."""
    out = fock_.contiguous().clone()
    f = as_device_f64(fock_hf, out.device).contiguous()
    check(_lib.load().gdft_fock_add_hf(_ptr(out), _ptr(f), out.shape[-1], float(clip), _stream(out.device)))
    return out


def coulomb(eri, rdm1, h1e=None, nuclear_repulsion=0.0, want_energy=False):
    dev = rdm1.device if isinstance(rdm1, torch.Tensor) and rdm1.is_cuda else require_cuda()
    rdm1 = as_device_f64(rdm1, dev)
    eri = as_device_f64(eri, dev)
    n = rdm1.shape[-1]
    if eri.shape != (n, n, n, n):
        raise ValueError(f"rep_tensor must be ({n}, {n}, {n}, {n}), got {tuple(eri.shape)}")
    vj = torch.empty((n, n), dtype=F64, device=dev)
    e = torch.empty((), dtype=F64, device=dev) if want_energy else None
    h = as_device_f64(h1e, dev) if want_energy else None
    check(_lib.load().gdft_coulomb(n, _ptr(eri), _ptr(rdm1), _ptr(h), float(nuclear_repulsion), _ptr(vj), _ptr(e),
                                   _stream(dev)))
    return vj, e
