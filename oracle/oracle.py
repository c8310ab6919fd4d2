"""FP64 CPU restatement of Grad DFT's XC grid path (test infrastructure only).

This module is the oracle the CUDA path is checked against.  It restates the
reference's arithmetic in torch float64 on the CPU, keeping the reference's
evaluation order, clip semantics (``jnp.clip(x, a_min=c)`` → gradient 0 below
``c``; ``abs_clip`` = ``where(|x| > t, x, 0)``), log2/exp2 forms and
``where`` masks.  ``torch.autograd`` stands in for ``jax.value_and_grad``.

Each function cites the reference file:line it follows (paths relative to the
GradDFT project root).  The restatement was pinned against fixtures produced
by running the reference's own ``grad_dft`` source (see
``tests/golden/make_golden.py``).
"""
from __future__ import annotations

import math
from typing import Optional

import numpy as np
import torch

F64 = torch.float64
CLIP = 1e-30

__all__ = [
    "abs_clip", "density", "grad_density", "lapl_density", "kinetic_density",
    "lsda_x_e", "b88_x_e", "pw92_c_e", "vwn_c_e", "lyp_c_e",
    "exchange_polarization_correction", "correlation_polarization_correction",
    "dm21_coefficient_inputs", "dm21_densities", "dm21_combine_cinputs", "dm21_combine_densities",
    "densities_generic", "dm21_network", "FUNCTIONALS", "energy_densities", "xc_energy",
    "xc_energy_and_grads", "xc_hvp", "predict_fock", "t64", "features_numpy", "FZETA_PP0",
    "hf_energy_density", "hf_density_grad_2_fock", "b3lyp_predict_with_chi", "dm21_hf_fock_terms",
    "DM21_GGA_COEFFS", "DM21_MGGA_COEFFS", "DENS_GGA_COEFFS", "DENS_MGGA_COEFFS",
]


def t64(x) -> torch.Tensor:
    if isinstance(x, torch.Tensor):
        return x.detach().to(dtype=F64, device="cpu")
    return torch.as_tensor(np.asarray(x), dtype=F64)


# --------------------------------------------------------------------------
# molecule.py
# --------------------------------------------------------------------------
def abs_clip(arr, threshold):
    """molecule.py:687-689."""
    return torch.where(arr.abs() > threshold, arr, torch.zeros((), dtype=arr.dtype))


def density(rdm1, ao):
    """molecule.py:385-409: rho_s(r) = sum_ab D_sab phi_ra phi_rb -> (grid, spin)."""
    return torch.einsum("sab,ra,rb->rs", rdm1, ao, ao)


def grad_density(rdm1, ao, grad_ao):
    """molecule.py:411-440: 2 sum_ab D_sab phi_ra d_j phi_rb -> (grid, spin, 3)."""
    return 2 * torch.einsum("sab,ra,rbj->rsj", rdm1, ao, grad_ao)


def lapl_density(rdm1, ao, grad_ao, grad2_ao):
    """molecule.py:442-474 (grad2_ao holds the diagonal second derivatives)."""
    return 2 * torch.einsum("sab,raj,rbj->rs", rdm1, grad_ao, grad_ao) + 2 * torch.einsum(
        "sab,ra,rbi->rs", rdm1, ao, grad2_ao
    )


def kinetic_density(rdm1, grad_ao):
    """molecule.py:476-502: 1/2 sum_j sum_ab D_sab d_j phi_a d_j phi_b -> (grid, spin)."""
    return 0.5 * torch.einsum("sab,raj,rbj->rs", rdm1, grad_ao, grad_ao)


# --------------------------------------------------------------------------
# functional.py: spin-polarisation corrections
# --------------------------------------------------------------------------
def exchange_polarization_correction(e_PF, rho):
    """functional.py:950-979 (Ullrich eq. 2.71)."""
    zeta = (rho[:, 0] - rho[:, 1]) / rho.sum(axis=1)

    def fzeta(z):
        return ((1 - z) ** (4 / 3) + (1 + z) ** (4 / 3) - 2) / (2 * (2 ** (1 / 3) - 1))

    return e_PF[:, 0] + (e_PF[:, 1] - e_PF[:, 0]) * fzeta(zeta)


def _fzeta_log2(z):
    zm = 2 ** (4 * torch.log2(1 - z) / 3)
    zp = 2 ** (4 * torch.log2(1 + z) / 3)
    return (zm + zp - 2) / (2 * (2 ** (1 / 3) - 1))


def _fzeta_second_derivative_at_zero() -> float:
    """functional.py:1040 ``grad(grad(fzeta))(0.0)`` evaluated by autodiff."""
    z = torch.zeros((), dtype=F64, requires_grad=True)
    f = _fzeta_log2(z)
    (g,) = torch.autograd.grad(f, z, create_graph=True)
    (h,) = torch.autograd.grad(g, z)
    return float(h)


FZETA_PP0 = _fzeta_second_derivative_at_zero()


def correlation_polarization_correction(e_tilde_PF, rho, clip_cte=CLIP):
    """functional.py:982-1045 (Ullrich eq. 2.75, PW92 alpha_c)."""
    log_rho = torch.log2(torch.clamp(rho.sum(axis=1), min=clip_cte))
    log_rs = math.log2((3 / (4 * math.pi)) ** (1 / 3)) - log_rho / 3.0
    zeta = torch.where(rho.sum(axis=1) > clip_cte, (rho[:, 0] - rho[:, 1]) / (rho.sum(axis=1)),
                       torch.zeros((), dtype=F64))
    A_ = 0.016887
    alpha1 = 0.11125
    beta1 = 10.357
    beta2 = 3.6231
    beta3 = 0.88026
    beta4 = 0.49671
    ars = 2 ** (math.log2(alpha1) + log_rs)
    brs_1_2 = 2 ** (math.log2(beta1) + log_rs / 2)
    brs = 2 ** (math.log2(beta2) + log_rs)
    brs_3_2 = 2 ** (math.log2(beta3) + 3 * log_rs / 2)
    brs2 = 2 ** (math.log2(beta4) + 2 * log_rs)
    alphac = 2 * A_ * (1 + ars) * torch.log(1 + (1 / (2 * A_)) / (brs_1_2 + brs + brs_3_2 + brs2))
    fz = _fzeta_log2(zeta)
    z4 = zeta ** 4
    return (e_tilde_PF[:, 0] + alphac * (fz / FZETA_PP0) * (1 - z4)
            + (e_tilde_PF[:, 1] - e_tilde_PF[:, 0]) * fz * z4)


# --------------------------------------------------------------------------
# popular_functionals.py
# --------------------------------------------------------------------------
def lsda_x_e(rho, clip_cte=CLIP):
    """popular_functionals.py:29-50."""
    rho = torch.clamp(rho, min=clip_cte)
    lda_es = (-3.0 / 4.0 * (torch.tensor([[3.0, 6.0]], dtype=F64) / math.pi) ** (1 / 3)
              * (rho.sum(axis=1, keepdims=True)) ** (4 / 3))
    return exchange_polarization_correction(lda_es, rho)


def b88_x_e(rho, grad_rho, clip_cte=CLIP):
    """popular_functionals.py:52-103 (B88 gradient correction only)."""
    beta = 0.0042
    rho = torch.clamp(rho, min=clip_cte)
    log_rho = torch.log2(torch.clamp(rho, min=clip_cte))
    grad_rho_norm_sq = torch.sum(grad_rho ** 2, axis=-1)
    log_grad_rho_norm = torch.log2(torch.clamp(grad_rho_norm_sq, min=clip_cte)) / 2
    log_x_sigma = log_grad_rho_norm - 4 / 3.0 * log_rho
    x_sigma = 2 ** log_x_sigma
    return -(beta * 2 ** (4 * log_rho / 3 + 2 * log_x_sigma
                          - torch.log2(1 + 6 * beta * x_sigma * torch.asinh(x_sigma)))).sum(axis=1)


_PW_A = torch.tensor([[0.031091, 0.015545]], dtype=F64)
_PW_ALPHA1 = torch.tensor([[0.21370, 0.20548]], dtype=F64)
_PW_BETA1 = torch.tensor([[7.5957, 14.1189]], dtype=F64)
_PW_BETA2 = torch.tensor([[3.5876, 6.1977]], dtype=F64)
_PW_BETA3 = torch.tensor([[1.6382, 3.3662]], dtype=F64)
_PW_BETA4 = torch.tensor([[0.49294, 0.62517]], dtype=F64)


def pw92_c_e(rho, clip_cte=CLIP):
    """popular_functionals.py:105-139."""
    log_rho = torch.log2(torch.clamp(rho.sum(axis=1, keepdims=True), min=clip_cte))
    log_rs = math.log2((3 / (4 * math.pi)) ** (1 / 3)) - log_rho / 3.0
    brs_1_2 = 2 ** (log_rs / 2 + torch.log2(_PW_BETA1))
    ars = 2 ** (log_rs + torch.log2(_PW_ALPHA1))
    brs = 2 ** (log_rs + torch.log2(_PW_BETA2))
    brs_3_2 = 2 ** (3 * log_rs / 2 + torch.log2(_PW_BETA3))
    brs2 = 2 ** (2 * log_rs + torch.log2(_PW_BETA4))
    e_PF = -2 * _PW_A * (1 + ars) * torch.log(1 + (1 / (2 * _PW_A)) / (brs_1_2 + brs + brs_3_2 + brs2))
    e_tilde = correlation_polarization_correction(e_PF, rho, clip_cte)
    return e_tilde * rho.sum(axis=1)


def vwn_c_e(rho, clip_cte=CLIP):
    """popular_functionals.py:141-195."""
    A = torch.tensor([[0.0621814, 0.0621814 / 2]], dtype=F64)
    b = torch.tensor([[3.72744, 7.06042]], dtype=F64)
    c = torch.tensor([[12.9352, 18.0578]], dtype=F64)
    x0 = torch.tensor([[-0.10498, -0.325]], dtype=F64)
    rho = torch.where(rho > clip_cte, rho, torch.zeros((), dtype=F64))
    log_rho = torch.log2(torch.clamp(rho.sum(axis=1, keepdims=True), min=clip_cte))
    log_rs = math.log2((3 / (4 * math.pi)) ** (1 / 3)) - log_rho / 3.0
    log_x = log_rs / 2
    x = 2 ** log_x
    X = 2 ** (2 * log_x) + 2 ** (log_x + torch.log2(b)) + c
    X0 = x0 ** 2 + b * x0 + c
    Q = torch.sqrt(4 * c - b ** 2)
    e_PF = (A / 2 * (2 * torch.log(x) - torch.log(X) + 2 * b / Q * torch.atan(Q / (2 * x + b))
                     - b * x0 / X0 * (torch.log((x - x0) ** 2 / X)
                                      + 2 * (2 * x0 + b) / Q * torch.atan(Q / (2 * x + b)))))
    e_tilde = correlation_polarization_correction(e_PF, rho, clip_cte)
    return e_tilde * rho.sum(axis=1)


def lyp_c_e(rho, grad_rho, grad2rho, clip_cte=CLIP):
    """popular_functionals.py:197-269 (original LYP, needs the Laplacian)."""
    a, b, c, d = 0.04918, 0.132, 0.2533, 0.349
    CF = (3 / 10) * (3 * math.pi ** 2) ** (2 / 3)
    rho = torch.clamp(rho, min=clip_cte)
    grad_rho_norm_sq = torch.sum(grad_rho ** 2, axis=-1)
    zero = torch.zeros((), dtype=F64)
    t = (torch.where(rho > clip_cte, grad_rho_norm_sq / rho, zero) - grad2rho) / 8.0
    frac = torch.where(rho.sum(axis=1) > clip_cte, ((rho ** 2).sum(axis=1)) / (rho.sum(axis=1)) ** 2,
                       torch.ones((), dtype=F64))
    gamma = 2 * (1 - frac)
    rhos_ts = rho.sum(axis=1) * t.sum(axis=1)
    rho_t = (rho * t).sum(axis=1)
    rho_grad2rho = (rho * grad2rho).sum(axis=1)
    rhom1_3 = (rho.sum(axis=1)) ** (-1 / 3)
    rho8_3 = (rho ** (8 / 3)).sum(axis=1)
    rhom5_3 = (rho.sum(axis=1)) ** (-5 / 3)
    exp_factor = torch.where(rho.sum(axis=1) > 0, torch.exp(-c * rhom1_3), zero)
    parenthesis = 2 ** (2 / 3) * CF * (rho8_3) - rhos_ts + rho_t / 9 + rho_grad2rho / 18
    braket_m_rho = torch.where(rho.sum(axis=1) > clip_cte, 2 * b * rhom5_3 * parenthesis * exp_factor, zero)
    return -a * torch.where(rho.sum(axis=1) > clip_cte,
                            gamma / (1 + d * rhom1_3) * (rho.sum(axis=1) + braket_m_rho), zero)


# --------------------------------------------------------------------------
# functional.py: DM21 features and network
# --------------------------------------------------------------------------
def dm21_coefficient_inputs(rho, grad_rho, tau, clip_cte=CLIP):
    """functional.py:504-531: 7 local features per grid point."""
    rho = torch.maximum(abs(rho), torch.tensor(clip_cte, dtype=F64)) * torch.sign(rho)
    grad_rho_norm = torch.sum(grad_rho ** 2, axis=-1)
    grad_rho_norm_sumspin = torch.sum(grad_rho.sum(axis=1, keepdims=True) ** 2, axis=-1)
    return torch.cat((rho, grad_rho_norm_sumspin, grad_rho_norm, tau), axis=1)


def _uw_ranges(functional_type):
    """functional.py:575-585 (and :1089-1099).  A dict {'u_range', 'w_range'} takes the meaning the
    docstring gives it (:548-556); the reference's code itself binds the ranges only for strings, so a
    dict raises UnboundLocalError there (recorded by tests/golden/make_golden.py)."""
    if isinstance(functional_type, dict):
        return functional_type["u_range"], functional_type["w_range"]
    if functional_type in ("LDA", "DM21"):
        return range(0, 1), range(0, 1)
    if functional_type == "GGA":
        return range(0, 2), range(0, 1)
    if functional_type == "MGGA":
        return range(0, 2), range(0, 2)
    raise ValueError(f"Functional type {functional_type} not recognized, must be one of LDA, GGA, MGGA.")


def dm21_densities(rho, grad_rho, tau, functional_type="LDA", clip_cte=CLIP):
    """functional.py:534-626."""
    beta = 1 / 1024.0
    u_range, w_range = _uw_ranges(functional_type)
    grad_rho_norm_sq = torch.sum(grad_rho ** 2, axis=-1)
    log_rho = torch.log2(torch.clamp(rho, min=clip_cte))
    log_grad_rho_norm = torch.log2(torch.clamp(grad_rho_norm_sq, min=clip_cte)) / 2
    log_x_sigma = log_grad_rho_norm - 4 / 3.0 * log_rho
    zero = torch.zeros((), dtype=F64)
    log_u_sigma = torch.where(torch.greater(log_rho, math.log2(clip_cte)),
                              log_x_sigma - torch.log2(1 + beta * (2 ** log_x_sigma)) + math.log2(beta), zero)
    log_tau = torch.log2(torch.clamp(tau, min=clip_cte))
    log_1t_sigma = -(5 / 3.0 * log_rho - log_tau + 2 / 3.0 * math.log2(6 * math.pi ** 2) + math.log2(3 / 5.0))
    log_w_sigma = torch.where(torch.greater(log_rho, math.log2(clip_cte)),
                              log_1t_sigma - torch.log2(1 + beta * (2 ** log_1t_sigma)) + math.log2(beta), zero)
    cols = []
    for i in u_range:
        for j in w_range:
            scale = -2 * math.pi * (3 / (4 * math.pi)) ** (4 / 3) if (i == 0 and j == 0) else 1.0
            cols.append((2 ** (4 / 3.0 * log_rho + i * log_u_sigma + j * log_w_sigma)).sum(axis=1, keepdims=True)
                        * scale)
    return torch.cat(cols, axis=1)


def dm21_combine_cinputs(cinputs, ehf):
    """functional.py:628-649: append ehf[:,0].T, ehf[:,1].T (omega-major per spin)."""
    return torch.cat([cinputs, ehf[:, 0].T, ehf[:, 1].T], axis=1)


def dm21_combine_densities(densities, ehf):
    """functional.py:652-675: append sum over spin of ehf for each omega."""
    return torch.cat([densities] + [ehf[i].sum(axis=0, keepdims=True).T for i in range(len(ehf))], axis=1)


def densities_generic(rho, grad_rho, tau, functional_type="LDA", clip_cte=CLIP):
    """functional.py:1048-1202 (generic exchange + PW92-based correlation features)."""
    beta = 1 / 1024.0
    u_range, w_range = _uw_ranges(functional_type)
    zero = torch.zeros((), dtype=F64)
    grad_rho_norm_sq = torch.sum(grad_rho ** 2, axis=-1)
    log_rho = torch.log2(torch.clamp(rho, min=clip_cte))
    log_grad_rho_norm = torch.log2(torch.clamp(grad_rho_norm_sq, min=clip_cte)) / 2
    log_x_sigma = log_grad_rho_norm - 4 / 3.0 * log_rho
    log_u_sigma = torch.where(torch.greater(log_rho, math.log2(clip_cte)),
                              log_x_sigma - torch.log2(1 + beta * (2 ** log_x_sigma)) + math.log2(beta), zero)
    log_tau = torch.log2(torch.clamp(tau, min=clip_cte))
    log_1t_sigma = log_tau - 5 / 3.0 * log_rho
    log_w_sigma = torch.where(torch.greater(log_rho, math.log2(clip_cte)),
                              log_1t_sigma - torch.log2(1 + beta * (2 ** log_1t_sigma)) + math.log2(beta), zero)
    cols = []
    for i in u_range:
        for j in w_range:
            cols.append(2 ** (4 / 3.0 * log_rho + i * log_u_sigma + j * log_w_sigma))
    grad_rho_norm_sq_ss = torch.sum((grad_rho.sum(axis=1)) ** 2, axis=-1)
    log_grad_rho_norm_ss = torch.log2(torch.clamp(grad_rho_norm_sq_ss, min=clip_cte)) / 2
    log_rho_ss = torch.log2(torch.clamp(rho.sum(axis=1), min=clip_cte))
    log_x_ss = log_grad_rho_norm_ss - 4 / 3.0 * log_rho_ss
    log_u_ss = torch.where(torch.greater(log_rho_ss, math.log2(clip_cte)),
                           log_x_ss - torch.log2(1 + beta * (2 ** log_x_ss)) + math.log2(beta), zero)
    log_u_ab = torch.where(torch.greater(log_rho_ss, math.log2(clip_cte)),
                           log_x_ss - 1 - torch.log2(1 + beta * (2 ** (log_x_ss - 1))) + math.log2(beta), zero)
    log_u_c = torch.stack((log_u_ss, log_u_ab), axis=1)
    log_tau_ss = torch.log2(torch.clamp(tau.sum(axis=1), min=clip_cte))
    log_1t_ss = log_tau_ss - 5 / 3.0 * log_rho_ss
    log_w_ss = torch.where(torch.greater(log_rho.sum(axis=1), math.log2(clip_cte)),
                           log_1t_ss - torch.log2(1 + beta * (2 ** log_1t_ss)) + math.log2(beta), zero)
    log_w_ab = torch.where(torch.greater(log_rho.sum(axis=1), math.log2(clip_cte)),
                           log_1t_ss - 1 - torch.log2(1 + beta * (2 ** (log_1t_ss - 1))) + math.log2(beta), zero)
    log_w_c = torch.stack((log_w_ss, log_w_ab), axis=1)
    log_rho1 = torch.log2(torch.clamp(rho.sum(axis=1, keepdims=True), min=clip_cte))
    log_rs = math.log2((3 / (4 * math.pi)) ** (1 / 3)) - log_rho1 / 3.0
    brs_1_2 = 2 ** (log_rs / 2 + torch.log2(_PW_BETA1))
    ars = 2 ** (log_rs + torch.log2(_PW_ALPHA1))
    brs = 2 ** (log_rs + torch.log2(_PW_BETA2))
    brs_3_2 = 2 ** (3 * log_rs / 2 + torch.log2(_PW_BETA3))
    brs2 = 2 ** (2 * log_rs + torch.log2(_PW_BETA4))
    # jnp.round(x, int(log10(1e-30))) rounds to a multiple of 1e30 (functional.py:1188-1191).
    e_PW92 = torch.round(-2 * _PW_A * (1 + ars) * torch.log(1 + (1 / (2 * _PW_A)) / (brs_1_2 + brs + brs_3_2 + brs2))
                         * 10.0 ** int(math.log10(clip_cte))) / 10.0 ** int(math.log10(clip_cte))
    for i in u_range:
        for j in w_range:
            cols.append(torch.where(torch.greater(e_PW92, clip_cte),
                                    2 ** (torch.log2(e_PW92) + i * log_u_c + j * log_w_c), zero))
    return torch.cat(cols, axis=1)


def _layer_norm(x, scale, bias, eps=1e-6):
    """flax.linen.LayerNorm defaults (epsilon 1e-6, var = E[x^2] - E[x]^2 clipped at 0)."""
    mean = x.mean(axis=-1, keepdims=True)
    mean2 = (x * x).mean(axis=-1, keepdims=True)
    var = torch.clamp(mean2 - mean * mean, min=0.0)
    return (x - mean) * torch.rsqrt(var + eps) * scale + bias


def dm21_network(params: dict, x, n_layers: int | None = None, squash_offset=1e-4, sigmoid_scale_factor=2.0):
    """functional.py:797-822 (DM21.default_nn) + NeuralFunctional.head (:407-419).

    n_layers defaults to the number of LayerNorm modules in params (6 for
    DM21's layer_widths)."""
    p = params["params"] if "params" in params else params
    if n_layers is None:
        n_layers = sum(1 for k in p if k.startswith("LayerNorm_"))
    if x.ndim == 1:  # canonicalize_inputs, functional.py:934-945
        x = x[:, None]
    x = torch.log(torch.abs(x) + squash_offset)
    x = x @ p["Dense_0"]["kernel"] + p["Dense_0"]["bias"]
    x = torch.tanh(x)
    for i in range(n_layers):
        res = x
        x = x @ p[f"Dense_{i + 1}"]["kernel"] + p[f"Dense_{i + 1}"]["bias"]
        x = x + res
        x = _layer_norm(x, p[f"LayerNorm_{i}"]["scale"], p[f"LayerNorm_{i}"]["bias"])
        x = torch.nn.functional.elu(x)
    x = x @ p[f"Dense_{n_layers + 1}"]["kernel"] + p[f"Dense_{n_layers + 1}"]["bias"]
    x = torch.sigmoid(x / sigmoid_scale_factor)
    return torch.squeeze(sigmoid_scale_factor * x)


# --------------------------------------------------------------------------
# Functionals (popular_functionals.py:271-393) and the energy (functional.py:160-342)
# --------------------------------------------------------------------------
B3LYP_COEFFS = [1 - 0.2, 0.72, 1 - 0.81, 0.81, 0.2]  # popular_functionals.py:336-343
# Test coefficients of the feature-power functionals (any constant rows serve; these mix signs).
DM21_GGA_COEFFS = [0.9, 1.1]
DM21_MGGA_COEFFS = [1.0, 0.5, -0.3, 0.2]
DENS_GGA_COEFFS = [-0.7, -0.6, 0.3, 0.2, 0.5, 0.4, 0.3, 0.2]
DENS_MGGA_COEFFS = [-0.7, -0.6, 0.3, 0.2, -0.2, -0.1, 0.1, 0.05, 0.5, 0.4, 0.3, 0.2, 0.1, 0.1, 0.1, 0.1]

FUNCTIONALS = {
    # name: (energy-density columns, constant coefficient row or None for neural)
    "LSDA": (("lsda",), [1.0]),
    "B88": (("lsda", "b88"), [1.0]),
    "VWN": (("vwn",), [1.0]),
    "LYP": (("lyp",), [1.0]),
    "PW92": (("pw92",), [1.0]),
    "BLYP": (("lsda", "b88", "lyp"), [1.0]),
    "B3LYP": (("lsda", "b88", "vwn", "lyp", "hf"), B3LYP_COEFFS),
    "DM21": (("dm21_lda", "hf_w0", "hf_w1"), None),
    # Constant-coefficient functionals on the feature powers of dm21_densities / densities
    # (functional.py:534-626, 1048-1202), selected as energy_densities=partial(..., functional_type=...).
    "DM21_GGA": ((("dm21", "GGA"),), DM21_GGA_COEFFS),
    "DM21_MGGA": ((("dm21", "MGGA"),), DM21_MGGA_COEFFS),
    "DENS_GGA": ((("dens", "GGA"),), DENS_GGA_COEFFS),
    "DENS_MGGA": ((("dens", "MGGA"),), DENS_MGGA_COEFFS),
}


def _features(rdm1, ao, grad_ao, grad2_ao):
    rho = density(rdm1, ao)
    grad_rho = grad_density(rdm1, ao, grad_ao)
    lapl = lapl_density(rdm1, ao, grad_ao, grad2_ao) if grad2_ao is not None else None
    tau = kinetic_density(rdm1, grad_ao)
    return rho, grad_rho, lapl, tau


def energy_densities(name, rho, grad_rho, lapl, tau, ehf=None, clip_cte=CLIP, clip_output=True):
    """Stack the energy-density columns of a named functional, then abs_clip (functional.py:160-185).

    ``clip_output=False`` leaves out the final abs_clip: the columns as
    ``energy_densities`` returns them before compute_densities clips them.
    """
    cols, _ = FUNCTIONALS[name]
    out = []
    for c in cols:
        if c == "lsda":
            out.append(lsda_x_e(rho, clip_cte))
        elif c == "b88":
            out.append(b88_x_e(rho, grad_rho, clip_cte))
        elif c == "vwn":
            out.append(vwn_c_e(rho, clip_cte))
        elif c == "lyp":
            out.append(lyp_c_e(rho, grad_rho, lapl, clip_cte))
        elif c == "pw92":
            out.append(pw92_c_e(rho, clip_cte))
        elif c == "hf":  # b3lyp_combine (popular_functionals.py:328-334), stop-gradient
            out.append(ehf.detach().sum(axis=(0, 1)))
        elif c == "dm21_lda":
            out.append(dm21_densities(rho, grad_rho, tau, "LDA", clip_cte)[:, 0])
        elif c == "hf_w0":
            out.append(ehf.detach()[0].sum(axis=0))
        elif c == "hf_w1":
            out.append(ehf.detach()[1].sum(axis=0))
        elif isinstance(c, tuple) and c[0] == "dm21":
            out.extend(dm21_densities(rho, grad_rho, tau, c[1], clip_cte).unbind(1))
        elif isinstance(c, tuple) and c[0] == "dens":
            out.extend(densities_generic(rho, grad_rho, tau, c[1], clip_cte).unbind(1))
        else:
            raise KeyError(c)
    stacked = torch.stack(out, axis=1)
    return abs_clip(stacked, clip_cte) if clip_output else stacked


def xc_energy(coefficients, densities, weights, clip_cte=CLIP):
    """functional.py:219-253 + _integrate (:316-342); broadcasting einsum as jnp does."""
    if coefficients.shape[0] == 1:
        coefficients = coefficients.expand(densities.shape[0], coefficients.shape[1])
    if coefficients.shape[1] == 1:
        coefficients = coefficients.expand(densities.shape[0], densities.shape[1])
    e = torch.einsum("rf,rf->r", coefficients, densities)
    e = abs_clip(e, clip_cte)
    return torch.einsum("r,r->", abs_clip(weights, clip_cte), abs_clip(e, clip_cte))


def _energy(name, rdm1, ao, grad_ao, grad2_ao, weights, params=None, ehf=None, clip_cte=CLIP):
    rho, grad_rho, lapl, tau = _features(rdm1, ao, grad_ao, grad2_ao)
    dens = energy_densities(name, rho, grad_rho, lapl, tau, ehf, clip_cte)
    _, coeffs = FUNCTIONALS[name]
    if coeffs is None:
        cin = dm21_coefficient_inputs(rho, grad_rho, tau)
        cin = dm21_combine_cinputs(cin, ehf.detach())
        c = dm21_network(params, cin)
        if c.ndim == 1:
            c = c[None, :]
    else:
        c = torch.tensor([coeffs], dtype=F64)
    return xc_energy(c, dens, weights, clip_cte)


def _tree_leaves(params):
    p = params["params"] if "params" in params else params
    leaves = []
    for k in sorted(p):
        for kk in sorted(p[k]):
            leaves.append((k, kk))
    return p, leaves


def xc_energy_and_grads(name, rdm1, ao, grad_ao, grad2_ao, weights, params=None, ehf=None,
                        want_param_grads=False, clip_cte=CLIP):
    """train.py:86-121 ``xc_energy_and_grads``: (E_xc, dE_xc/dD[, dE_xc/dtheta])."""
    D = t64(rdm1).clone().requires_grad_(True)
    ao, grad_ao = t64(ao), t64(grad_ao)
    grad2_ao = None if grad2_ao is None else t64(grad2_ao)
    weights = t64(weights)
    ehf = None if ehf is None else t64(ehf)
    tparams = None
    leaves = []
    if params is not None:
        p, names = _tree_leaves(params)
        tparams = {"params": {k: {} for k in p}}
        for k, kk in names:
            t = t64(p[k][kk]).clone().requires_grad_(want_param_grads)
            tparams["params"][k][kk] = t
            leaves.append(((k, kk), t))
    E = _energy(name, D, ao, grad_ao, grad2_ao, weights, tparams, ehf, clip_cte)
    inputs = [D] + ([t for _, t in leaves] if want_param_grads else [])
    grads = torch.autograd.grad(E, inputs, allow_unused=True)
    V = grads[0]
    if not want_param_grads:
        return float(E.detach()), V.numpy()
    dparams = {}
    for ((k, kk), _), g in zip(leaves, grads[1:]):
        dparams.setdefault(k, {})[kk] = (torch.zeros_like(_) if g is None else g).numpy()
    return float(E.detach()), V.numpy(), {"params": dparams}


def xc_hvp(name, rdm1, ao, grad_ao, grad2_ao, weights, tangent, params=None, ehf=None, clip_cte=CLIP):
    """Second-order adjoint of ``xc_energy_and_grads``: with L = <G, dE_xc/dD> (G = ``tangent``),
    return (L, dL/dD, dL/dtheta).  This is what jax.grad computes when it differentiates through a
    Fock matrix built from V_xc, as in the differentiable SCF loop (evaluate.py:314-344)."""
    D = t64(rdm1).clone().requires_grad_(True)
    G = t64(tangent)
    ao, grad_ao = t64(ao), t64(grad_ao)
    grad2_ao = None if grad2_ao is None else t64(grad2_ao)
    weights = t64(weights)
    ehf = None if ehf is None else t64(ehf)
    tparams, leaves = None, []
    if params is not None:
        p, names = _tree_leaves(params)
        tparams = {"params": {k: {} for k in p}}
        for k, kk in names:
            t = t64(p[k][kk]).clone().requires_grad_(True)
            tparams["params"][k][kk] = t
            leaves.append(((k, kk), t))
    E = _energy(name, D, ao, grad_ao, grad2_ao, weights, tparams, ehf, clip_cte)
    (V,) = torch.autograd.grad(E, D, create_graph=True)
    L = (V * G).sum()
    grads = torch.autograd.grad(L, [D] + [t for _, t in leaves], allow_unused=True)
    dparams = {}
    for ((k, kk), t), g in zip(leaves, grads[1:]):
        dparams.setdefault(k, {})[kk] = (torch.zeros_like(t) if g is None else g).detach().numpy()
    return float(L.detach()), grads[0].detach().numpy(), ({"params": dparams} if leaves else None)


def predict_fock(E_xc, V_xc, h1e, vj, nonxc_energy, clip_cte=CLIP):
    """train.py:147-163: F = abs_clip(1/2 (F + F^T)) with F = abs_clip(h1e + J + V_xc)."""
    V = t64(V_xc)
    fock = t64(h1e)[None] + t64(vj) + V if t64(vj).ndim == 2 else t64(h1e) + t64(vj) + V
    fock = abs_clip(fock, clip_cte)
    fock = 0.5 * (fock + fock.transpose(1, 2))
    fock = abs_clip(fock, clip_cte)
    return E_xc + nonxc_energy, abs_clip(fock, clip_cte).numpy()


# --------------------------------------------------------------------------
# Exact exchange from a chi tensor (molecule.py:153-300, 504-685; train.py:165-213)
# --------------------------------------------------------------------------
def hf_energy_density(rdm1, ao, chi):
    """molecule.py:507-541: ehf (omega, spin, grid) = -1/2 einsum("rwsc,sac,ra->wsr", chi, rdm1, ao)."""
    return -0.5 * torch.einsum("rwsc,sac,ra->wsr", t64(chi), t64(rdm1), t64(ao))


def hf_density_grad_2_fock(name, rdm1, ao, grad_ao, grad2_ao, weights, chi, ehf, clip_cte=CLIP):
    """molecule.py:545-613 for a constant-coefficient functional: (omega, spin, n, n).

    gr = d xc_energy / d ehf with the densities as predict passes them
    (energy_densities unclipped, train.py:167-178, combined with ehf by
    b3lyp_combine); F[w,s,a,b] = -1/2 sum_r chi[r,w,s,b] gr[w,s,r] ao[r,a].
    """
    cols, coeffs = FUNCTIONALS[name]
    with torch.no_grad():
        rho, grad_rho, lapl, tau = _features(t64(rdm1), t64(ao), t64(grad_ao),
                                             None if grad2_ao is None else t64(grad2_ao))
        raw = energy_densities(name, rho, grad_rho, lapl, tau, t64(ehf), clip_cte, clip_output=False)
    ehf_v = t64(ehf).clone().requires_grad_(True)
    dens = torch.cat([raw[:, :-1], ehf_v.sum(axis=(0, 1))[:, None]], axis=1)
    E = xc_energy(torch.tensor([coeffs], dtype=F64), dens, t64(weights), clip_cte)
    (gr,) = torch.autograd.grad(E, ehf_v)
    return -0.5 * torch.einsum("rwsb,wsr,ra->wsab", t64(chi), gr, t64(ao))


def dm21_hf_fock_terms(rdm1, ao, grad_ao, grad2_ao, weights, params, chi, clip_cte=CLIP):
    """dm21_hfgrads_densities and dm21_hfgrads_cinputs (functional.py:677-757), omegas 0 and 0.4.

    (F_dens, F_cin), each (spin, n, n) summed over omega: the HF Fock terms
    with dE/d ehf taken through the HF energy-density columns (the network's
    inputs held) and through the HF inputs (the densities held), with the
    local densities unclipped as predict passes them.
    """
    with torch.no_grad():
        rho, grad_rho, _, tau = _features(t64(rdm1), t64(ao), t64(grad_ao), None if grad2_ao is None else t64(grad2_ao))
        ehf = hf_energy_density(rdm1, ao, chi)
        dens_wout = dm21_densities(rho, grad_rho, tau, "LDA", clip_cte)
        cin_wout = dm21_coefficient_inputs(rho, grad_rho, tau, clip_cte)
    w = t64(weights)
    p = params["params"] if "params" in params else params
    params = {"params": {k: {kk: t64(v) for kk, v in d.items()} for k, d in p.items()}}
    e1 = ehf.clone().requires_grad_(True)
    c1 = dm21_network(params, dm21_combine_cinputs(cin_wout, ehf)).detach()
    (g_dens,) = torch.autograd.grad(xc_energy(c1, dm21_combine_densities(dens_wout, e1), w, clip_cte), e1)
    e2 = ehf.clone().requires_grad_(True)
    c2 = dm21_network(params, dm21_combine_cinputs(cin_wout, e2))
    (g_cin,) = torch.autograd.grad(xc_energy(c2, dm21_combine_densities(dens_wout, ehf), w, clip_cte), e2)
    fock = lambda g: -0.5 * torch.einsum("rwsb,wsr,ra->sab", t64(chi), g, t64(ao))  # noqa: E731
    return fock(g_dens), fock(g_cin)


def b3lyp_predict_with_chi(rdm1, ao, grad_ao, grad2_ao, weights, h1e, eri, chi, omegas, nuclear_repulsion,
                           clip_cte=CLIP):
    """energy_predictor(B3LYP) (train.py:124-218) with its HF terms from chi: (E, F)."""
    i0 = list(np.asarray(omegas)).index(0.0)
    ehf0 = hf_energy_density(rdm1, ao, t64(chi)[:, i0:i0 + 1])
    e, v = xc_energy_and_grads("B3LYP", rdm1, ao, grad_ao, grad2_ao, weights, ehf=ehf0, clip_cte=clip_cte)
    d = np.asarray(rdm1).sum(0)
    vj = np.einsum("pqrt,rt->pq", eri, d)
    enonxc = nuclear_repulsion + np.einsum("ij,ij->", d, h1e) + np.einsum("pq,pq->", d, vj) / 2.0
    E, F = predict_fock(e, v, h1e, vj, enonxc, clip_cte)
    vexpl = hf_density_grad_2_fock("B3LYP", rdm1, ao, grad_ao, grad2_ao, weights, t64(chi)[:, i0:i0 + 1], ehf0,
                                   clip_cte).sum(0)
    F = t64(F) + vexpl + vexpl.transpose(1, 2)
    return E, abs_clip(F, clip_cte).detach().numpy()


def features_numpy(rdm1, ao, grad_ao, grad2_ao):
    """rho (N,2), grad_rho (N,2,3), lapl (N,2), tau (N,2) as numpy float64."""
    with torch.no_grad():
        r = _features(t64(rdm1), t64(ao), t64(grad_ao), None if grad2_ao is None else t64(grad2_ao))
    return tuple(None if x is None else x.numpy() for x in r)
