"""A torch-float64 stand-in for the parts of jax/flax that Grad DFT's XC path uses.

Fixture generation only (see ``make_golden.py``).  JAX, flax, optax, orbax,
jaxtyping and typeguard are not installed in this environment, so this module
registers small replacements in ``sys.modules`` that follow the documented
semantics of the calls the reference makes on the XC path:

* ``jax.numpy``: elementwise math, ``einsum`` (with size-1 broadcasting),
  ``where``/``clip``/``maximum``, reductions with ``axis``/``keepdims``, and
  ``round(x, decimals)`` as ``round_half_even(x * 10**d) / 10**d``;
* ``jax.grad``/``jax.value_and_grad`` over tensors and dict pytrees via
  ``torch.autograd`` (``create_graph=True`` so they nest);
* ``jax.lax.stop_gradient`` as ``detach``;
* ``flax.struct.dataclass`` as a frozen dataclass with ``replace``;
* ``flax.linen.Module.apply`` with flax's auto-naming of ``Dense_k`` and
  ``LayerNorm_k`` submodules and flax defaults (Dense: ``x @ kernel + bias``;
  LayerNorm: epsilon 1e-6, ``var = max(0, E[x^2] - E[x]^2)``,
  ``y = (x - mean) * (rsqrt(var + eps) * scale) + bias``).

Everything is float64 (the reference runs with ``jax_enable_x64``).
"""
from __future__ import annotations

import dataclasses
import enum
import functools
import math
import sys
import types
import typing

import numpy as np
import torch

F64 = torch.float64


def _t(x):
    if isinstance(x, torch.Tensor):
        return x
    if isinstance(x, bool):
        return torch.tensor(x)
    if isinstance(x, (int, float)):
        return torch.tensor(float(x), dtype=F64)
    a = np.asarray(x)
    if a.dtype.kind == "f":
        return torch.as_tensor(a.astype(np.float64))
    return torch.as_tensor(a)


def _axis(axis):
    return tuple(axis) if isinstance(axis, (list, tuple)) else axis


class _DType:
    """A jnp scalar type: usable as a dtype and callable (jnp.int64(x))."""

    def __init__(self, dt):
        self.torch = dt

    def __call__(self, x):
        return torch.as_tensor(x).to(self.torch)


def _dt(d):
    return d.torch if isinstance(d, _DType) else d


class _At:
    """x.at[idx].set(v) as a copy; updates at out-of-bounds indices are dropped, as JAX drops them."""

    def __init__(self, t):
        self.t = t

    def __getitem__(self, idx):
        t = self.t

        class _Set:
            @staticmethod
            def set(v):
                out = t.clone()
                try:
                    out[idx] = _t(v).to(out.dtype) if isinstance(v, torch.Tensor) else v
                except IndexError:
                    pass
                return out

        return _Set()


def _mk_jnp():
    m = types.ModuleType("jax.numpy")
    m.pi = math.pi
    m.inf = math.inf
    m.float64 = F64
    m.float32 = torch.float32
    m.int64 = _DType(torch.int64)
    m.int32 = _DType(torch.int32)
    m.ndarray = torch.Tensor

    def array(x, dtype=None):
        t = _t(x) if not isinstance(x, (list, tuple)) or not any(isinstance(e, torch.Tensor) for e in x) \
            else torch.stack([_t(e) for e in x])
        if dtype is not None:
            t = t.to(_dt(dtype))
        elif t.is_floating_point():
            t = t.to(F64)
        return t

    m.array = array
    m.asarray = array
    for name, fn in dict(log2=torch.log2, log=torch.log, exp=torch.exp, sqrt=torch.sqrt, tanh=torch.tanh,
                         arctan=torch.atan, arcsinh=torch.asinh, abs=torch.abs, sign=torch.sign,
                         isnan=torch.isnan, isinf=torch.isinf).items():
        setattr(m, name, (lambda f: (lambda x: f(_t(x))))(fn))

    def clip(a, a_min=None, a_max=None, min=None, max=None):  # noqa: A002
        # jnp.clip is maximum(a_min, x) then minimum(a_max, .): at an exact tie the gradient is split in
        # half, as torch.maximum / torch.minimum split it (torch.clamp would pass all of it).
        lo = a_min if a_min is not None else min
        hi = a_max if a_max is not None else max
        x = _t(a)
        if lo is not None:
            x = torch.maximum(x, torch.as_tensor(lo, dtype=x.dtype))
        if hi is not None:
            x = torch.minimum(x, torch.as_tensor(hi, dtype=x.dtype))
        return x

    m.clip = clip

    def where(c, x=None, y=None):
        if not isinstance(c, torch.Tensor):
            return _t(x) if bool(c) else _t(y)
        x, y = _t(x), _t(y)
        if x.dtype != y.dtype:
            dt = torch.promote_types(x.dtype, y.dtype)
            x, y = x.to(dt), y.to(dt)
        return torch.where(c, x, y)

    m.where = where
    m.maximum = lambda a, b: torch.maximum(_t(a), _t(b))
    m.minimum = lambda a, b: torch.minimum(_t(a), _t(b))
    m.greater = lambda a, b: torch.greater(_t(a), _t(b))
    m.less = lambda a, b: torch.less(_t(a), _t(b))
    m.logical_and = lambda a, b: torch.logical_and(_t(a), _t(b))

    m.eye = lambda n, dtype=None: torch.eye(int(n), dtype=F64)
    if not hasattr(m, "dot"):
        m.dot = lambda a, b: torch.matmul(_t(a), _t(b))
    m.any = lambda x, axis=None: torch.any(_t(x)) if axis is None else torch.any(_t(x), dim=axis)
    m.isclose = lambda a, b, rtol=1e-05, atol=1e-08, equal_nan=False: torch.isclose(
        _t(a).to(F64), _t(b).to(F64), rtol=rtol, atol=atol, equal_nan=equal_nan)

    def einsum(subscripts, *ops, precision=None, **_):
        ts = [_t(o) for o in ops]
        if any(t.is_complex() for t in ts):  # jnp.einsum promotes mixed real/complex operands
            ts = [t if t.is_complex() else t.to(torch.complex128) for t in ts]
        return torch.einsum(subscripts, *ts)

    m.einsum = einsum

    def _sum(x, axis=None, keepdims=False):
        x = _t(x)
        if axis is None:
            return x.sum()
        return torch.sum(x, dim=_axis(axis), keepdim=keepdims)

    m.sum = _sum
    m.concatenate = lambda xs, axis=0: torch.cat([_t(x) for x in xs], dim=axis)
    m.stack = lambda xs, axis=0: torch.stack([_t(x) for x in xs], dim=axis)
    m.expand_dims = lambda x, axis: torch.unsqueeze(_t(x), axis)

    def squeeze(x, axis=None):
        x = _t(x)
        return torch.squeeze(x) if axis is None else torch.squeeze(x, axis)

    m.squeeze = squeeze

    def _round(x, decimals=0):
        x = _t(x)
        if decimals == 0:
            return torch.round(x)
        factor = 10 ** decimals
        return torch.round(x * factor) / factor

    m.round = _round
    m.empty = lambda shape, dtype=F64: torch.empty(shape, dtype=_dt(dtype) if dtype is not None else F64)
    m.zeros = lambda shape, dtype=F64: torch.zeros(shape, dtype=_dt(dtype) if dtype is not None else F64)
    m.ones = lambda shape, dtype=F64: torch.ones(shape, dtype=_dt(dtype) if dtype is not None else F64)
    m.zeros_like = lambda x: torch.zeros_like(_t(x))
    m.identity = lambda n, dtype=F64: torch.eye(n, dtype=_dt(dtype))
    m.diag = lambda x: torch.diag(_t(x))
    m.diag_indices_from = lambda x: (torch.arange(_t(x).shape[0]), torch.arange(_t(x).shape[0]))
    m.divide = lambda a, b: torch.div(_t(a), _t(b))
    m.multiply = lambda a, b: torch.mul(_t(a), _t(b))
    m.nan_to_num = lambda x: torch.nan_to_num(_t(x))
    m.moveaxis = lambda x, a, b: torch.movedim(_t(x), a, b)
    m.less_equal = lambda a, b: torch.less_equal(_t(a), _t(b))
    m.vectorize = lambda f, signature=None: f  # called on single matrices here
    m.dot = lambda a, b, precision=None: _t(a) @ _t(b)
    m.tensordot = lambda a, b, axes=2, precision=None: torch.tensordot(_t(a), _t(b), dims=axes)
    m.reshape = lambda x, shape: torch.reshape(_t(x), shape)
    m.argsort = lambda x: torch.argsort(_t(x))
    m.linalg = types.SimpleNamespace(norm=lambda x: torch.linalg.norm(_t(x)), inv=torch.linalg.inv,
                                     eigh=torch.linalg.eigh, cholesky=torch.linalg.cholesky,
                                     qr=lambda x: torch.linalg.qr(_t(x)))
    return m


def _tree_prepare(x):
    """Make every tensor leaf of a pytree differentiable; return (tree, leaves, rebuild)."""
    if isinstance(x, dict):
        keys = list(x.keys())
        parts = [_tree_prepare(x[k]) for k in keys]
        leaves = [leaf for _, ls, _ in parts for leaf in ls]

        def rebuild(gs, parts=parts, keys=keys):
            out, i = {}, 0
            for k, (_, ls, rb) in zip(keys, parts):
                out[k] = rb(gs[i:i + len(ls)])
                i += len(ls)
            return out

        return {k: p[0] for k, p in zip(keys, parts)}, leaves, rebuild
    t = _t(x)
    if not (t.is_floating_point() or t.is_complex()):
        t = t.to(F64)
    if not t.requires_grad:
        t = t.detach().clone().requires_grad_(True)
    return t, [t], (lambda gs: gs[0])


def value_and_grad(fun, argnums=0, has_aux=False):
    nums = argnums if isinstance(argnums, (tuple, list)) else (argnums,)

    @functools.wraps(fun)
    def wrapped(*args, **kwargs):
        with torch.enable_grad():
            return _vg_call(fun, nums, argnums, has_aux, args, kwargs)

    return wrapped


def _vg_call(fun, nums, argnums, has_aux, args, kwargs):
    args = list(args)
    if True:
        rebuilds, leaves_all, counts = [], [], []
        for i in nums:
            tree, leaves, rb = _tree_prepare(args[i])
            args[i] = tree
            rebuilds.append(rb)
            leaves_all += leaves
            counts.append(len(leaves))
        out = fun(*args, **kwargs)
        val = out[0] if has_aux else out
        gs = torch.autograd.grad(val, leaves_all, create_graph=True, allow_unused=True)
        gs = [torch.zeros_like(l) if g is None else g for g, l in zip(gs, leaves_all)]
        # jax.grad of a real function of a complex leaf is dL/dRe - i dL/dIm, the
        # conjugate of the gradient torch returns
        gs = [g.conj() if g.is_complex() else g for g in gs]
        res, j = [], 0
        for rb, c in zip(rebuilds, counts):
            res.append(rb(gs[j:j + c]))
            j += c
        g = tuple(res) if isinstance(argnums, (tuple, list)) else res[0]
        return (out, g)


def grad(fun, argnums=0, has_aux=False):
    vg = value_and_grad(fun, argnums, has_aux)

    @functools.wraps(fun)
    def wrapped(*args, **kwargs):
        out, g = vg(*args, **kwargs)
        return (g, out[1]) if has_aux else g

    return wrapped


def _identity_decorator(f=None, *a, **k):
    if f is None or not callable(f):
        return lambda g: g
    return f


class _Precision(enum.Enum):
    DEFAULT = 0
    HIGH = 1
    HIGHEST = 2


# ---------------------------------------------------------------- flax shim
_CTX: list = []


class Module:
    def apply(self, variables, *args, **kwargs):
        params = variables.get("params", {}) if isinstance(variables, dict) else {}
        _CTX.append({"params": params, "counts": {}})
        try:
            if hasattr(type(self), "setup"):
                self.setup()
            return self.__call__(*args, **kwargs)
        finally:
            _CTX.pop()

    def sow(self, *args, **kwargs):
        return None


def _auto_name(kind):
    ctx = _CTX[-1]
    k = ctx["counts"].get(kind, 0)
    ctx["counts"][kind] = k + 1
    return f"{kind}_{k}"


class Dense:
    def __init__(self, features, param_dtype=None, kernel_init=None, bias_init=None, use_bias=True, **_):
        self.features = features
        self.use_bias = use_bias
        self.name = _auto_name("Dense")

    def __call__(self, x):
        p = _CTX[-1]["params"][self.name]
        y = torch.tensordot(_t(x), _t(p["kernel"]), dims=([x.ndim - 1], [0]))
        if self.use_bias:
            y = y + _t(p["bias"])
        return y


class LayerNorm:
    def __init__(self, epsilon=1e-6, param_dtype=None, use_bias=True, use_scale=True, **_):
        self.epsilon = epsilon
        self.use_bias = use_bias
        self.use_scale = use_scale
        self.name = _auto_name("LayerNorm")

    def __call__(self, x):
        p = _CTX[-1]["params"][self.name]
        mean = x.mean(dim=-1, keepdim=True)
        mean2 = (x * x).mean(dim=-1, keepdim=True)
        var = torch.clamp(mean2 - mean * mean, min=0.0)
        mul = torch.rsqrt(var + self.epsilon)
        if self.use_scale:
            mul = mul * _t(p["scale"])
        y = (x - mean) * mul
        if self.use_bias:
            y = y + _t(p["bias"])
        return y


def _struct_dataclass(cls=None, **kw):
    def wrap(c):
        c = dataclasses.dataclass(frozen=True)(c)
        c.replace = lambda self, **k: dataclasses.replace(self, **k)
        return c

    return wrap if cls is None else wrap(cls)


class _Sub:
    """jaxtyping-style ``Float[Array, "..."]`` placeholder."""

    def __getitem__(self, item):
        return typing.Any


class _CustomVjp:
    """jax.custom_vjp: the primal runs as is; with defvjp, a torch.autograd.Function calls bwd(res, g)."""

    def __init__(self, f):
        self.f, self.fwd, self.bwd = f, None, None

    def defvjp(self, fwd, bwd):
        self.fwd, self.bwd = fwd, bwd

    def __call__(self, *args):
        tensors = [a for a in args if isinstance(a, torch.Tensor)]
        if self.fwd is None or not torch.is_grad_enabled() or not any(t.requires_grad for t in tensors):
            return self.f(*args)
        outer = self

        class _Fn(torch.autograd.Function):
            @staticmethod
            def forward(ctx, *a):
                out, res = outer.fwd(*a)
                ctx.res = res
                return tuple(out) if isinstance(out, (tuple, list)) else out

            @staticmethod
            def backward(ctx, *gs):
                ref = ctx.res[0] if isinstance(ctx.res, tuple) else None
                gs = tuple(torch.zeros_like(r) if g is None else g
                           for g, r in zip(gs, ref if isinstance(ref, tuple) else gs))
                return outer.bwd(ctx.res, gs if len(gs) > 1 else gs[0])

        return _Fn.apply(*args)


def vmap(fun, in_axes=0, out_axes=0, **_):
    """jax.vmap for single-array outputs: a loop over the mapped axis, then a stack."""

    def wrapped(*args):
        axes = tuple(in_axes) if isinstance(in_axes, (tuple, list)) else (in_axes,) * len(args)
        n = next(_t(a).shape[ax] for a, ax in zip(args, axes) if ax is not None)
        outs = []
        for i in range(n):
            sl = [_t(a).select(ax, i) if ax is not None else a for a, ax in zip(args, axes)]
            outs.append(_t(fun(*sl)))
        return torch.stack(outs, dim=out_axes)

    return wrapped


_orig_getitem = torch.Tensor.__getitem__


def _clamped_getitem(self, idx):
    """Indexing that clamps out-of-bounds integer indices, as JAX's gathers do."""
    try:
        return _orig_getitem(self, idx)
    except IndexError:
        parts = idx if isinstance(idx, tuple) else (idx,)
        if not all(isinstance(p, (int, slice)) for p in parts):
            raise
        fixed = tuple(min(max(p, -self.shape[d]), self.shape[d] - 1) if isinstance(p, int) else p
                      for d, p in enumerate(parts))
        return _orig_getitem(self, fixed)


def install():
    """Register the stand-in modules (idempotent)."""
    torch.Tensor.at = property(lambda self: _At(self))
    torch.Tensor.__getitem__ = _clamped_getitem
    torch.Tensor.astype = lambda self, dt: self.to(_dt(dt))
    if "jax" in sys.modules and getattr(sys.modules["jax"], "_is_graddft_shim", False):
        return
    jax = types.ModuleType("jax")
    jax._is_graddft_shim = True
    jnp = _mk_jnp()
    jax.numpy = jnp
    lax = types.ModuleType("jax.lax")
    lax.Precision = _Precision
    lax.stop_gradient = lambda x: _t(x).detach() if isinstance(x, torch.Tensor) else x

    def fori_loop(lo, hi, body=None, init=None, body_fun=None, init_val=None):
        body = body if body is not None else body_fun
        v = init if init is not None else init_val
        for i in range(lo, hi):
            v = body(i, v)
        return v

    lax.fori_loop = fori_loop
    def cond(p, t, f, *operands, operand=None):
        args = operands if operands else (operand,)
        return t(*args) if bool(p) else f(*args)

    lax.cond = cond
    jax.lax = lax
    jax.grad = grad
    jax.value_and_grad = value_and_grad

    def jit(f=None, **kw):
        if f is None:
            return lambda g: g
        return f

    jax.jit = jit

    jax.vmap = vmap
    jax.custom_vjp = _CustomVjp
    jax.config = types.SimpleNamespace(x64_enabled=True, update=lambda *a, **k: None)
    prof = types.ModuleType("jax.profiler")
    prof.annotate_function = lambda f=None, name=None, **k: (f if f is not None else (lambda g: g))
    jax.profiler = prof
    jnn = types.ModuleType("jax.nn")
    jnn.sigmoid = torch.sigmoid
    jnn.gelu = torch.nn.functional.gelu
    jnn.elu = lambda x, alpha=1.0: torch.nn.functional.elu(x, alpha)
    inits = types.ModuleType("jax.nn.initializers")
    inits.zeros = lambda *a, **k: None
    inits.he_normal = lambda *a, **k: (lambda *aa, **kk: None)
    jnn.initializers = inits
    jax.nn = jnn
    rnd = types.ModuleType("jax.random")
    rnd.normal = lambda *a, **k: None
    rnd.PRNGKey = lambda *a, **k: None
    jax.random = rnd
    jsp = types.ModuleType("jax.scipy")
    jax.scipy = jsp
    tu = types.ModuleType("jax.tree_util")
    tu.tree_map = lambda f, t: {k: tu.tree_map(f, v) for k, v in t.items()} if isinstance(t, dict) else f(t)
    tu.tree_leaves = lambda t: [l for v in t.values() for l in tu.tree_leaves(v)] if isinstance(t, dict) else [t]
    jax.tree_util = tu
    for name, mod in {"jax": jax, "jax.numpy": jnp, "jax.lax": lax, "jax.profiler": prof, "jax.nn": jnn,
                      "jax.nn.initializers": inits, "jax.random": rnd, "jax.scipy": jsp,
                      "jax.tree_util": tu}.items():
        sys.modules[name] = mod

    flax = types.ModuleType("flax")
    struct = types.ModuleType("flax.struct")
    struct.dataclass = _struct_dataclass
    linen = types.ModuleType("flax.linen")
    linen.Module = Module
    linen.compact = lambda f: f
    linen.Dense = Dense
    linen.LayerNorm = LayerNorm
    core = types.ModuleType("flax.core")
    core.freeze = lambda x: x
    core.unfreeze = lambda x: x
    training = types.ModuleType("flax.training")
    ts = types.ModuleType("flax.training.train_state")
    ts.TrainState = type("TrainState", (), {})
    training.train_state = ts
    training.checkpoints = types.SimpleNamespace()
    flax.struct, flax.linen, flax.core, flax.training = struct, linen, core, training
    for name, mod in {"flax": flax, "flax.struct": struct, "flax.linen": linen, "flax.core": core,
                      "flax.training": training, "flax.training.train_state": ts}.items():
        sys.modules[name] = mod

    optax = types.ModuleType("optax")
    optax.OptState = object
    optax.GradientTransformation = object
    optax.apply_updates = lambda p, u: p + u

    class _Adam:
        """optax.adam (scale_by_adam with bias correction, then scale by -learning_rate), for the
        orbital-optimiser fixtures; optax itself is not installed."""

        def __init__(self, learning_rate, b1=0.9, b2=0.999, eps=1e-8, eps_root=0.0):
            self.lr, self.b1, self.b2, self.eps, self.eps_root = learning_rate, b1, b2, eps, eps_root

        def init(self, params):
            return (0, torch.zeros_like(params), torch.zeros_like(params))

        def update(self, grads, state, params=None):
            count, mu, nu = state
            mu = self.b1 * mu + (1 - self.b1) * grads
            nu = self.b2 * nu + (1 - self.b2) * grads * grads
            count += 1
            mu_hat, nu_hat = mu / (1 - self.b1 ** count), nu / (1 - self.b2 ** count)
            return -self.lr * mu_hat / (torch.sqrt(nu_hat + self.eps_root) + self.eps), (count, mu, nu)

    optax.adam = _Adam
    orbax = types.ModuleType("orbax")
    ock = types.ModuleType("orbax.checkpoint")
    ock.Checkpointer = object
    ock.PyTreeCheckpointer = lambda *a, **k: None
    orbax.checkpoint = ock
    jt = types.ModuleType("jaxtyping")
    for n in ("Array", "PyTree", "Scalar", "PRNGKeyArray"):
        setattr(jt, n, typing.Any)
    for n in ("Float", "Int", "Complex", "Bool"):
        setattr(jt, n, _Sub())
    jt.jaxtyped = _identity_decorator
    tg = types.ModuleType("typeguard")
    tg.typechecked = _identity_decorator
    for name, mod in {"optax": optax, "orbax": orbax, "orbax.checkpoint": ock, "jaxtyping": jt,
                      "typeguard": tg}.items():
        sys.modules[name] = mod


def load_reference(root: str, with_solid: bool = False):
    """Execute the reference's molecule/functional/popular_functionals/train modules.

    ``grad_dft/__init__.py`` is not executed (it imports PySCF, h5py and the
    SCF machinery); a package object is assembled instead and the four source
    files are executed from ``root`` unchanged.
    """
    import importlib.util
    import os

    install()
    pkg = types.ModuleType("grad_dft")
    pkg.__path__ = []
    sys.modules["grad_dft"] = pkg
    utils = types.ModuleType("grad_dft.utils")
    utils.__path__ = []

    def vmap_chunked(fun, in_axes=0, out_axes=0, chunk_size=None, **_):
        return vmap(fun, in_axes=in_axes, out_axes=out_axes)

    utils.vmap_chunked = vmap_chunked
    sys.modules["grad_dft.utils"] = utils
    types_mod = types.ModuleType("grad_dft.utils.types")
    types_mod.DType = typing.Any
    types_mod.default_dtype = lambda: F64
    types_mod.Hartree2kcalmol = 627.50947
    sys.modules["grad_dft.utils.types"] = types_mod
    utils.types = types_mod

    def run(name):
        path = os.path.join(root, "grad_dft", name + ".py")
        spec = importlib.util.spec_from_file_location("grad_dft." + name, path)
        mod = importlib.util.module_from_spec(spec)
        sys.modules["grad_dft." + name] = mod
        spec.loader.exec_module(mod)
        return mod

    mol = run("molecule")
    for n in ("Grid", "Molecule", "abs_clip", "make_rdm1", "orbital_grad", "density", "grad_density",
              "coulomb_energy"):
        setattr(pkg, n, getattr(mol, n))

    if with_solid:
        sol = run("solid")
        pkg.Solid, pkg.KPointInfo = sol.Solid, sol.KPointInfo
    else:
        class Solid:  # the periodic path is left out unless asked for
            pass

        pkg.Solid = Solid
        sol = None
    fun = run("functional")
    for n in ("DispersionFunctional", "Functional", "NeuralFunctional", "DM21",
              "correlation_polarization_correction", "exchange_polarization_correction",
              "canonicalize_inputs", "dm21_coefficient_inputs", "dm21_densities", "densities",
              "dm21_combine_cinputs", "dm21_combine_densities"):
        setattr(pkg, n, getattr(fun, n))
    pop = run("popular_functionals")
    train = run("train")
    pkg.energy_predictor = train.energy_predictor
    return types.SimpleNamespace(molecule=mol, functional=fun, popular=pop, train=train, solid=sol)


def load_scf(root: str, ref):
    """Execute utils/eigenproblem.py and evaluate.py (the SCF loops) on top of load_reference.

    evaluate.py's PySCF-facing imports (interface/pyscf.py, scipy-style
    optimizers) are not used by the differentiable loops and get stand-ins.
    """
    import importlib.util
    import os

    def run(name, fname):
        spec = importlib.util.spec_from_file_location(name, os.path.join(root, "grad_dft", fname))
        mod = importlib.util.module_from_spec(spec)
        sys.modules[name] = mod
        spec.loader.exec_module(mod)
        return mod

    jsc = types.ModuleType("jax.scipy")
    jsc.special = types.SimpleNamespace(erfc=torch.special.erfc)
    jsc.optimize = types.SimpleNamespace(minimize=None)
    sys.modules["jax.scipy"], sys.modules["jax.scipy.special"] = jsc, jsc.special
    sys.modules["jax.scipy.optimize"] = jsc.optimize
    sys.modules["jax"].scipy = jsc
    iface = types.ModuleType("grad_dft.interface")
    iface.__path__ = []
    pys = types.ModuleType("grad_dft.interface.pyscf")
    pys.generate_chi_tensor = None
    # scf_loop builds PySCF objects up front only to regenerate chi when the molecule has omegas
    # (evaluate.py:404-408, 509-521); without omegas placeholders do
    pys.mol_from_Molecule = lambda molecule, *a, **k: None
    pys.process_mol = lambda *a, **k: (None, None)
    sys.modules["grad_dft.interface"], sys.modules["grad_dft.interface.pyscf"] = iface, pys
    eig = run("grad_dft.utils.eigenproblem", "utils/eigenproblem.py")
    utils = sys.modules["grad_dft.utils"]
    utils.Optimizer = typing.Any
    for n in ("safe_eigh", "safe_general_eigh", "safe_fock_solver"):
        setattr(utils, n, getattr(eig, n))
    ev = run("grad_dft.evaluate", "evaluate.py")
    ref.eigenproblem, ref.evaluate = eig, ev
    return ev
