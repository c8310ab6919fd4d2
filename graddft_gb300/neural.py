"""NeuralFunctional and DM21 (functional.py:345-500, 676-932) on the fused device path.

A ``DM21`` here has the reference's plugin slots and defaults; its coefficient
network (``default_nn`` + ``head``) runs as the library's network kernels,
and ``xc_energy_and_grads`` / ``energy`` return E_xc with dE_xc/d rdm1 and
dE_xc/d theta from the hand-written adjoint.  Parameters are the flax tree
``{"params": {"Dense_k": {"kernel", "bias"}, "LayerNorm_k": {"scale", "bias"}}}``
(names as flax gives them to DM21.default_nn, functional.py:876-891), as torch
tensors, numpy arrays or DLPack producers.

The HF inputs (``nograd_densities`` / ``nograd_coefficient_inputs``) are
stop-gradient, as in the reference; with a chi tensor on the molecule they come
from ``Molecule.HF_energy_density`` and the explicit HF Fock terms
(``densitygrads`` / ``coefficient_input_grads``, train.py:200-213) are built
from the network's dE/d ehf (FP64 network form).
"""
from __future__ import annotations

import ctypes
import weakref
from dataclasses import dataclass, field
from typing import Any, Callable, Optional

import torch

from . import _lib, engine
from .functional import CLIP, Functional, dm21_combine_cinputs, dm21_combine_densities, dm21_densities
from .molecule import HF_GRAD_CLIP, Molecule

F64 = torch.float64


def _stop_grad_hf(atoms, *_, **__):
    """DM21's nograd HF inputs: Molecule.HF_energy_density([0.0, 0.4]) (functional.py:779-785)."""
    return atoms.HF_energy_density(torch.tensor([0.0, 0.4], dtype=F64))


def dm21_coefficient_inputs(atoms, clip_cte: float = CLIP, *_, **__):
    """functional.py:504-531: the 7 local DM21 features (grid, 7), computed on the device."""
    x, _ = _neural_inputs(atoms, _DEFAULT_NET, _zero_ehf(atoms))
    return x[:, :7]


def _zero_ehf(atoms):
    r = atoms.resident()
    return torch.zeros((2, 2, r.n_grid), dtype=F64, device=r.device)


def _neural_inputs(atoms, net: engine.Network, ehf):
    r = atoms.resident()
    ehf = engine.as_device_f64(ehf, r.device)
    if ehf is None or tuple(ehf.shape) != (2, 2, r.n_grid):
        raise ValueError(f"ehf must be (2, 2, {r.n_grid})")
    x = torch.empty((r.n_grid, net.n_in), dtype=F64, device=r.device)
    e = torch.empty((r.n_grid, net.n_out), dtype=F64, device=r.device)
    ws = r._neural_ws(net)
    _lib.check(_lib.load().gdft_neural_inputs(ctypes.byref(r.desc), engine._ptr(atoms._rdm1()), ctypes.byref(net.desc),
                                              engine._ptr(ehf), engine._ptr(x), engine._ptr(e), engine._ptr(ws),
                                              ws.numel(), engine._stream(r.device)))
    return x, e


def _omega_summed_hf_term(atoms, method, gradient, functional, params, omegas, ehf, *args):
    """sum over omega of atoms.<method>(functional, params, omegas, ehf, *args), as functional.py:677-757
    sum what the molecule returns.  With the library's own Molecule method the sum is one exchange
    contraction over all omegas (g and chi summed inside B) instead of one per omega."""
    own = all(getattr(type(atoms), m, None) is getattr(Molecule, m)
              for m in (method, "select_HF_omegas", "_hf_fock_per_omega", "_hf_fock_omega_sum"))
    if not own:  # a Molecule subclass that changes any step keeps its own per-omega method
        return getattr(atoms, method)(functional, params, omegas, ehf, *args).sum(dim=0)
    chi = atoms.select_HF_omegas(omegas)
    # The reference calls the molecule method without clip_cte (functional.py:711-713, 752-754), so the
    # method's default applies.
    g = getattr(functional, gradient)(params, atoms, engine.as_device_f64(ehf, atoms.device), HF_GRAD_CLIP)
    return atoms._hf_fock_omega_sum(chi, g)


def dm21_hfgrads_densities(functional, params, atoms, ehf, coefficient_inputs, densities_wout_hf,
                           omegas=(0.0, 0.4)):
    """functional.py:677-716: the HF Fock term from dE/d ehf through the HF densities, summed over omega
    (Molecule.HF_density_grad_2_Fock summed)."""
    return _omega_summed_hf_term(atoms, "HF_density_grad_2_Fock", "hf_density_gradient", functional, params,
                                 omegas, ehf, coefficient_inputs, densities_wout_hf)


def dm21_hfgrads_cinputs(functional, params, atoms, ehf, cinputs_wout_hf, densities, omegas=(0.0, 0.4)):
    """functional.py:718-757: the HF Fock term from dE/d ehf through the HF inputs, summed over omega
    (Molecule.HF_coefficient_input_grad_2_Fock summed)."""
    return _omega_summed_hf_term(atoms, "HF_coefficient_input_grad_2_Fock", "hf_cinput_gradient", functional,
                                 params, omegas, ehf, cinputs_wout_hf, densities)


# Both terms take dE_xc/d ehf from the functional's device pass (cached by xc_energy_and_grads); of
# their arguments they read ehf alone, and only when that pass has not run for the molecule.
dm21_hfgrads_densities._gdft_reads_ehf_only = True
dm21_hfgrads_cinputs._gdft_reads_ehf_only = True


class _NeuralXc(torch.autograd.Function):
    """E_xc(D, theta) with the hand-written adjoint: backward returns g * V_xc and g * dE/dtheta."""

    @staticmethod
    def forward(ctx, rdm1, flat, resident, net, ehf):
        exc, vxc, dp = resident.neural_xc_energy_and_grads(rdm1.detach(), net, flat.detach(), ehf,
                                                           want_vxc=ctx.needs_input_grad[0],
                                                           want_dparams=ctx.needs_input_grad[1])
        ctx.save_for_backward(*(t for t in (vxc, dp) if t is not None))
        ctx.has = (vxc is not None, dp is not None)
        return exc

    @staticmethod
    def backward(ctx, g):
        saved = list(ctx.saved_tensors)
        gv = g * saved.pop(0) if ctx.has[0] else None
        gp = g * saved.pop(0) if ctx.has[1] else None
        return gv, gp, None, None, None


class _NeuralXcPair(torch.autograd.Function):
    """(E_xc, V_xc)(D, theta), both differentiable.

    Backward: for cotangents (gE, gV), dD = gE V + d<gV, V>/dD and
    dtheta = gE dE/dtheta + d<gV, V>/dtheta, the second-order terms from the
    library's Hessian-vector product.  Nothing of the network pass is kept
    between forward and backward: the backward recomputes it (per-call
    checkpointing), so long unrolled loops hold only D, theta and V.
    """

    @staticmethod
    def forward(ctx, rdm1, flat, resident, net, ehf):
        ctx.set_materialize_grads(False)  # an output nothing reads has no cotangent: no second-order pass for it
        exc, vxc, dp = resident.neural_xc_energy_and_grads(rdm1.detach(), net, flat.detach(), ehf, want_vxc=True,
                                                           want_dparams=ctx.needs_input_grad[1])
        ctx.save_for_backward(rdm1.detach(), flat.detach(), vxc, *(t for t in (dp,) if t is not None))
        ctx.resident, ctx.net, ctx.ehf = resident, net, ehf
        return exc, vxc

    @staticmethod
    def backward(ctx, g_e, g_v):
        saved = ctx.saved_tensors
        rdm1, flat, vxc = saved[:3]
        dp = saved[3] if len(saved) > 3 else None
        d_rdm1 = d_flat = None
        want_d, want_p = ctx.needs_input_grad[0], ctx.needs_input_grad[1]
        if want_d:
            d_rdm1 = g_e * vxc if g_e is not None else torch.zeros_like(vxc)
        if want_p:
            d_flat = g_e * dp if g_e is not None else torch.zeros_like(flat)
        if g_v is not None:
            _, hd, hp = ctx.resident.neural_xc_hvp(rdm1, ctx.net, flat, ctx.ehf, g_v.contiguous(), want_value=False,
                                                   want_drdm1=want_d, want_dparams=want_p)
            if want_d:
                d_rdm1 = d_rdm1 + hd
            if want_p:
                d_flat = d_flat + hp
        return d_rdm1, d_flat, None, None, None


@dataclass
class NeuralFunctional(Functional):
    """functional.py:345-500: a Functional whose coefficients are a network.

    ``layer_widths`` / ``squash_offset`` / ``sigmoid_scale_factor`` /
    ``local_features`` describe the DM21.default_nn architecture, the one
    network this path builds (elu activation, LayerNorm epsilon 1e-6).
    """

    kernel_init: Any = None
    bias_init: Any = None
    activation: Any = "elu"
    param_dtype: Any = F64
    squash_offset: float = 1e-4
    layer_widths: tuple = (256, 256, 256, 256, 256, 256)
    local_features: int = 3
    sigmoid_scale_factor: float = 2.0
    n_input_features: int = 11
    # Arithmetic form of the network on the device: "fp64" (reference form) or
    # "tf32x3" (hidden-layer GEMMs on the tensor cores, FP32 activations).
    precision: str = "fp64"

    def network(self, clip_cte: float = CLIP) -> engine.Network:
        widths = set(self.layer_widths)
        if len(widths) != 1:
            raise NotImplementedError("layer_widths must all be equal (residual blocks)")
        if self.activation not in ("elu", getattr(torch.nn.functional, "elu")):
            raise NotImplementedError("the device network implements the elu activation of DM21")
        return engine.Network(n_layers=len(self.layer_widths), width=widths.pop(), n_in=self.n_input_features,
                              n_out=self.local_features, squash_offset=self.squash_offset,
                              sigmoid_scale=self.sigmoid_scale_factor, clip=clip_cte, precision=self.precision)

    # ---------------------------------------------------------- flax-like
    def init(self, rng=0, example_inputs=None):
        """Glorot-uniform parameters in the flax tree layout (seeded by an integer)."""
        from .synthetic import glorot_params

        seed = int(rng) if not isinstance(rng, torch.Generator) else int(rng.initial_seed())
        p = glorot_params(layer_widths=tuple(self.layer_widths), n_in=self.n_input_features,
                          n_out=self.local_features, seed=seed)
        return {"params": {k: {kk: torch.as_tensor(v) for kk, v in d.items()} for k, d in p["params"].items()}}

    def apply(self, params, coefficient_inputs, **kwargs):
        """The coefficients c_theta(x) (rows, local_features) on the device (functional.py:797-822, 407-419)."""
        engine.require_cuda()
        net = self.network()
        x = coefficient_inputs
        if not isinstance(x, torch.Tensor) or not x.is_cuda:
            x = engine.as_device_f64(x, engine.require_cuda())
        dev = x.device
        x = x.to(F64).contiguous()
        if x.ndim == 1:
            x = x[:, None]
        if x.ndim != 2 or x.shape[1] != net.n_in:
            raise ValueError(f"coefficient inputs must be (rows, {net.n_in}), got {tuple(x.shape)}")
        flat = net.flatten(params, dev)
        n = x.shape[0]
        wb = ctypes.c_size_t()
        _lib.check(_lib.load().gdft_network_apply_workspace_bytes(ctypes.byref(net.desc), n, ctypes.byref(wb)))
        ws = torch.empty(wb.value, dtype=torch.uint8, device=dev)
        c = torch.empty((n, net.n_out), dtype=F64, device=dev)
        _lib.check(_lib.load().gdft_network_apply(ctypes.byref(net.desc), engine._ptr(flat), n, engine._ptr(x),
                                                  engine._ptr(c), engine._ptr(ws), ws.numel(), engine._stream(dev)))
        return torch.squeeze(c)

    # ------------------------------------------------------------ the API
    def _ehf(self, atoms):
        ehf = None
        if self.nograd_coefficient_inputs is not None:
            ehf = self.nograd_coefficient_inputs(atoms)
        elif self.nograd_densities is not None:
            ehf = self.nograd_densities(atoms)
        if ehf is None:
            raise NotImplementedError("the device network takes the 4 stop-gradient HF inputs of DM21")
        return ehf

    def _check_slots(self):
        from .functional import energy_density_columns

        if self.energy_densities is not None and energy_density_columns(self.energy_densities) != (_lib.COL_DM21_LDA,):
            raise NotImplementedError("the device network pass takes dm21_densities' LDA column as its "
                                      "local energy density")
        if getattr(self.combine_inputs, "__name__", "") != "dm21_combine_cinputs" and self.combine_inputs is not None:
            raise NotImplementedError("combine_inputs must be dm21_combine_cinputs")
        if self.combine_densities is not None and getattr(self.combine_densities, "_gdft_hf_cols", None) is None:
            raise NotImplementedError("combine_densities must be dm21_combine_densities")

    def compute_coefficient_inputs(self, atoms, *args, **kwargs):
        """functional.py:187-217: (grid, 11) = local features + HF inputs."""
        self._check_slots()
        x, _ = _neural_inputs(atoms, self.network(), self._ehf(atoms))
        return x

    def compute_densities(self, atoms, clip_cte: float = CLIP, *args, **kwargs):
        """functional.py:160-185: abs_clip of [e_LDA, sum_s ehf(w0), sum_s ehf(w1)]."""
        self._check_slots()
        _, e = _neural_inputs(atoms, self.network(clip_cte), self._ehf(atoms))
        return torch.where(e.abs() > clip_cte, e, torch.zeros((), dtype=F64, device=e.device))

    def xc_energy(self, params, grid, coefficient_inputs, densities, clip_cte: float = CLIP, **kwargs):
        """functional.py:219-253: sum_r abs_clip(w) abs_clip(sum_f c_rf e_rf) with c = apply(params, inputs)."""
        c = self.apply(params, coefficient_inputs)
        if c.ndim == 1:
            c = c[None, :]
        dens = densities.to(F64)
        e = torch.einsum("rf,rf->r", c.expand_as(dens) if c.shape[0] == 1 else c, dens)
        w = engine.as_device_f64(grid.weights, dens.device)
        zero = torch.zeros((), dtype=F64, device=dens.device)
        e = torch.where(e.abs() > clip_cte, e, zero)
        w = torch.where(w.abs() > clip_cte, w, zero)
        return torch.dot(w, e)

    def xc_energy_and_grads(self, params, atoms, clip_cte: float = CLIP):
        """(E_xc, dE_xc/d rdm1) (train.py:86-121).

        With a chi tensor on the molecule and HF Fock terms to come (densitygrads /
        coefficient_input_grads), the same network pass also makes dE/d ehf for them.
        """
        hf_terms = self.densitygrads is not None or self.coefficient_input_grads is not None
        if hf_terms and getattr(atoms, "chi", None) is not None:
            self._check_slots()
            r = atoms.resident()
            net = self.network(clip_cte)
            e, v, g_dens, g_cin = r.neural_xc_hf_grads(atoms._rdm1(), net, net.flatten(params, r.device),
                                                       self._ehf(atoms), want_vxc=True)
            self.__dict__["_hf_cache"] = (self._hf_key(params, atoms, clip_cte), (g_dens, g_cin))
            return e, v
        e, v, _ = self.xc_energy_and_grads_params(params, atoms, clip_cte, want_dparams=False)
        return e, v

    def xc_energy_and_grads_params(self, params, atoms, clip_cte: float = CLIP, want_dparams: bool = True):
        """(E_xc, dE_xc/d rdm1, dE_xc/d theta as a flax tree) in one fused pass."""
        self._check_slots()
        r = atoms.resident()
        net = self.network(clip_cte)
        flat = net.flatten(params, r.device)
        exc, vxc, dp = r.neural_xc_energy_and_grads(atoms._rdm1(), net, flat, self._ehf(atoms), want_vxc=True,
                                                   want_dparams=want_dparams)
        return exc, vxc, (net.unflatten(dp) if dp is not None else None)

    def xc_energy_and_potential(self, params, atoms, clip_cte: float = CLIP):
        """(E_xc, V_xc), both differentiable in rdm1 and in the parameter tensors (to second order).

        What value_and_grad(argnums=1) of train.py:86 gives inside a jax.grad-ed
        program: the Fock matrices of an unrolled SCF loop are built from V_xc
        and differentiated through.
        """
        self._check_slots()
        r = atoms.resident()
        net = self.network(clip_cte)
        flat = net.flatten(params, r.device)
        rdm1 = atoms.rdm1 if isinstance(atoms.rdm1, torch.Tensor) and atoms.rdm1.requires_grad else atoms._rdm1()
        return _NeuralXcPair.apply(rdm1, flat, r, net, self._ehf(atoms))

    @staticmethod
    def _hf_key(params, atoms, clip_cte):
        rdm1 = atoms.rdm1
        ver = (rdm1.data_ptr(), rdm1._version) if isinstance(rdm1, torch.Tensor) else None
        return (weakref.ref(atoms), params, rdm1, ver, clip_cte)

    def _hf_cached(self, params, atoms, clip_cte):
        cached = self.__dict__.get("_hf_cache")
        if cached is None:
            return None
        (ref, p, rdm1, ver, clip), grads = cached
        now = self._hf_key(params, atoms, clip_cte)
        if ref() is atoms and p is params and rdm1 is atoms.rdm1 and ver == now[3] and clip == clip_cte:
            return grads
        return None

    def _hf_grads(self, params, atoms, ehf, clip_cte):
        """(g_dens, g_cin), reused from the xc pass of the same predict when it already made them."""
        self._check_slots()
        cached = self._hf_cached(params, atoms, clip_cte)
        if cached is not None:
            return cached
        r = atoms.resident()
        net = self.network(clip_cte)
        _, _, g_dens, g_cin = r.neural_xc_hf_grads(atoms._rdm1(), net, net.flatten(params, r.device), ehf)
        self.__dict__["_hf_cache"] = (self._hf_key(params, atoms, clip_cte), (g_dens, g_cin))
        return g_dens, g_cin

    def hf_density_gradient(self, params, atoms, ehf, clip_cte: float = CLIP):
        """dE_xc/d ehf (2, 2, grid) through the HF energy-density columns (molecule.py:598-603)."""
        return self._hf_grads(params, atoms, ehf, clip_cte)[0]

    def hf_cinput_gradient(self, params, atoms, ehf, clip_cte: float = CLIP):
        """dE_xc/d ehf (2, 2, grid) through the network's HF inputs (molecule.py:668-673)."""
        return self._hf_grads(params, atoms, ehf, clip_cte)[1]

    def energy_xc_only(self, params, atoms, *args, **kwargs):
        """E_xc as a differentiable torch scalar in rdm1 and in the parameter tensors."""
        self._check_slots()
        r = atoms.resident()
        net = self.network(kwargs.get("clip_cte", CLIP))
        flat = net.flatten(params, r.device)
        rdm1 = atoms.rdm1 if isinstance(atoms.rdm1, torch.Tensor) and atoms.rdm1.requires_grad else atoms._rdm1()
        return _NeuralXc.apply(rdm1, flat, r, net, self._ehf(atoms))


@dataclass
class DM21(NeuralFunctional):
    """functional.py:759-932 with the reference's defaults.

    As in the reference, the default ``densitygrads`` / ``coefficient_input_grads``
    need the chi tensor (energy_predictor raises ValueError without it); pass
    ``densitygrads=None, coefficient_input_grads=None`` and stop-gradient
    ``nograd_*`` inputs to use supplied HF energy densities instead.
    """

    coefficients: Callable = None
    energy_densities: Callable = dm21_densities
    nograd_densities: Optional[Callable] = _stop_grad_hf
    densitygrads: Optional[Callable] = dm21_hfgrads_densities
    combine_densities: Optional[Callable] = dm21_combine_densities
    coefficient_inputs: Optional[Callable] = dm21_coefficient_inputs
    nograd_coefficient_inputs: Optional[Callable] = _stop_grad_hf
    coefficient_input_grads: Optional[Callable] = dm21_hfgrads_cinputs
    combine_inputs: Optional[Callable] = dm21_combine_cinputs
    is_xc: bool = True


_DEFAULT_NET = engine.Network()
