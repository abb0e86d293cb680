"""Parameter update of the VMC optimisation step: Adam with the reference's learning-rate schedules.

The reference's standard optimiser (``optimization/opt_utils.py:73-76``,
``configuration.py:1091-1106``) is ``optax.adam(lr_schedule)``: b1 = 0.9, b2 = 0.999, eps = 1e-8,
eps_root = 0, learning rate 1e-3 on the inverse schedule (``opt_utils.py:40-50``,
``configuration.py:1073-1078``). Adam as published (Kingma and Ba), in optax's form: at update t
(counted from 0)
    m <- b1 m + (1 - b1) g,    v <- b2 v + (1 - b2) g^2,
    theta <- theta - lr(t) * (m / (1 - b1^(t+1))) / (sqrt(v / (1 - b2^(t+1))) + eps).
The update runs in place on the packed float32 parameter vector on the GPU, moments in float32
as the reference keeps them; the padding between packed tensors has zero gradient and stays zero.
After an update the derived weight copies are rebuilt (``Params.prepare``).
"""
from __future__ import annotations

import dataclasses
import math

import torch


@dataclasses.dataclass
class InverseLRSchedule:
    """lr(t) = base / (1 + (t + offset_time) / decay_time), at least `minimum`, times a linear
    warmup over `warmup` steps (opt_utils.py:40-50; defaults configuration.py:1073-1078)."""

    decay_time: float = 6000.0
    offset_time: float = 0.0
    warmup: int = 0
    minimum: float = 0.0

    def __call__(self, base: float, t: int) -> float:
        lr = base / (1.0 + (t + self.offset_time) / self.decay_time)
        lr = max(self.minimum, lr)
        if self.warmup > 0:
            lr *= min((t + 1) / self.warmup, 1.0)
        return lr


@dataclasses.dataclass
class ExponentialLRSchedule:
    """lr(t) = base exp(-(t + offset_time) / decay_time), at least `minimum`, linear warmup
    (opt_utils.py:51-60); defaults of ExponentialLRSchedule (configuration.py:1065-1070)."""

    decay_time: float = 10000.0
    offset_time: float = 0.0
    warmup: int = 0
    minimum: float = 0.0

    def __call__(self, base: float, t: int) -> float:
        lr = base * math.exp(-(t + self.offset_time) / self.decay_time)
        lr = max(self.minimum, lr)
        if self.warmup > 0:
            lr *= min((t + 1) / self.warmup, 1.0)
        return lr


@dataclasses.dataclass
class ConstantLRSchedule:
    """lr(t) = base (opt_utils.py:67-68)."""

    def __call__(self, base: float, t: int) -> float:
        return base


class Adam:
    """Adam over the packed parameter vector (optax.adam semantics, see the module docstring)."""

    def __init__(self, flat: torch.Tensor, learning_rate: float = 1e-3, schedule=None, b1: float = 0.9,
                 b2: float = 0.999, eps: float = 1e-8):
        self.learning_rate = float(learning_rate)
        self.schedule = schedule if schedule is not None else InverseLRSchedule()
        self.b1, self.b2, self.eps = float(b1), float(b2), float(eps)
        self.mu = torch.zeros_like(flat, dtype=torch.float32)
        self.nu = torch.zeros_like(flat, dtype=torch.float32)
        self.count = 0

    def update_(self, flat: torch.Tensor, grads: torch.Tensor) -> torch.Tensor:
        """One Adam update of `flat` in place with the gradient `grads` (same layout)."""
        g = grads.to(torch.float32)
        t = self.count
        self.mu.mul_(self.b1).add_(g, alpha=1.0 - self.b1)
        self.nu.mul_(self.b2).addcmul_(g, g, value=1.0 - self.b2)
        c1 = 1.0 - self.b1 ** (t + 1)
        c2 = 1.0 - self.b2 ** (t + 1)
        lr = self.schedule(self.learning_rate, t)
        denom = (self.nu / c2).sqrt_().add_(self.eps)
        flat.addcdiv_(self.mu, denom, value=-lr / c1)
        self.count = t + 1
        return flat

    def step(self, params, grads: torch.Tensor):
        """Updates a ``api.Params`` in place and rebuilds its derived weight copies."""
        self.update_(params.flat, grads)
        params.prepare()
        return params
