"""Gradient transformations with optax's protocol, for the orbital optimisers.

``mol_orb_optimizer`` (evaluate.py:595-780) takes an optax
``GradientTransformation`` ``tx``: ``state = tx.init(W)``,
``updates, state = tx.update(grads, state, W)``, ``W = apply_updates(W, updates)``.
Any object with that protocol on torch tensors works; ``adam`` and ``sgd``
follow optax's definitions of the published methods (Adam: Kingma and Ba,
ICLR 2015, with optax's defaults b1 = 0.9, b2 = 0.999, eps = 1e-8,
eps_root = 0 and bias correction).
"""
from __future__ import annotations

from dataclasses import dataclass

import torch


def apply_updates(params: torch.Tensor, updates: torch.Tensor) -> torch.Tensor:
    return params + updates


@dataclass
class _AdamState:
    count: int
    mu: torch.Tensor
    nu: torch.Tensor


class adam:  # noqa: N801 - optax's name
    def __init__(self, learning_rate: float, b1: float = 0.9, b2: float = 0.999, eps: float = 1e-8,
                 eps_root: float = 0.0):
        self.lr, self.b1, self.b2, self.eps, self.eps_root = float(learning_rate), b1, b2, eps, eps_root

    def init(self, params: torch.Tensor) -> _AdamState:
        return _AdamState(0, torch.zeros_like(params), torch.zeros_like(params))

    def update(self, grads: torch.Tensor, state: _AdamState, params=None):
        mu = self.b1 * state.mu + (1.0 - self.b1) * grads
        nu = self.b2 * state.nu + (1.0 - self.b2) * grads * grads
        count = state.count + 1
        mu_hat = mu / (1.0 - self.b1 ** count)
        nu_hat = nu / (1.0 - self.b2 ** count)
        updates = -self.lr * mu_hat / (torch.sqrt(nu_hat + self.eps_root) + self.eps)
        return updates, _AdamState(count, mu, nu)


class sgd:  # noqa: N801 - optax's name
    def __init__(self, learning_rate: float):
        self.lr = float(learning_rate)

    def init(self, params: torch.Tensor):
        return None

    def update(self, grads: torch.Tensor, state, params=None):
        return -self.lr * grads, state
