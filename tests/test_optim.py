"""Adam parameter update (no GPU): against a float64 restatement of the published algorithm in
optax's form (optax.adam as optimization/opt_utils.py:73-76 builds it) and the reference's
learning-rate schedules (opt_utils.py:40-68)."""
import math

import numpy as np
import pytest
import torch

from deeperwin_gb300 import optim


def _adam_reference(theta, grads, lr_fn, b1=0.9, b2=0.999, eps=1e-8):
    m = np.zeros_like(theta)
    v = np.zeros_like(theta)
    out = []
    for t, g in enumerate(grads):
        m = b1 * m + (1 - b1) * g
        v = b2 * v + (1 - b2) * g * g
        m_hat = m / (1 - b1 ** (t + 1))
        v_hat = v / (1 - b2 ** (t + 1))
        theta = theta - lr_fn(t) * m_hat / (np.sqrt(v_hat) + eps)
        out.append(theta.copy())
    return out


def test_inverse_schedule_defaults():
    s = optim.InverseLRSchedule()
    assert s(1e-3, 0) == 1e-3
    assert s(1e-3, 6000) == pytest.approx(5e-4)
    w = optim.InverseLRSchedule(decay_time=100.0, offset_time=10.0, warmup=4, minimum=2e-4)
    assert w(1e-3, 0) == pytest.approx(1e-3 / 1.1 * 0.25)
    assert w(1e-3, 100000) == pytest.approx(2e-4)
    e = optim.ExponentialLRSchedule(decay_time=50.0)
    assert e(1e-3, 50) == pytest.approx(1e-3 * math.exp(-1))
    assert optim.ConstantLRSchedule()(3e-4, 123) == 3e-4


@pytest.mark.parametrize("schedule", [optim.InverseLRSchedule(), optim.InverseLRSchedule(decay_time=3.0, warmup=2),
                                      optim.ConstantLRSchedule()])
def test_adam_matches_reference_algorithm(schedule):
    rng = np.random.default_rng(0)
    n = 1000
    theta0 = rng.standard_normal(n)
    grads = [rng.standard_normal(n) * (10.0 ** rng.uniform(-4, 1, n)) for _ in range(7)]
    grads[3][:50] = 0.0                                    # zero-gradient entries (packed padding)
    flat = torch.tensor(theta0, dtype=torch.float32)
    opt = optim.Adam(flat, learning_rate=1e-2, schedule=schedule)
    ref = _adam_reference(theta0.astype(np.float32).astype(np.float64), grads, lambda t: schedule(1e-2, t))
    for t, g in enumerate(grads):
        opt.update_(flat, torch.tensor(g, dtype=torch.float32))
        np.testing.assert_allclose(flat.numpy(), ref[t], rtol=1e-6, atol=1e-6)
    assert opt.count == 7


def test_padding_stays_fixed():
    flat = torch.zeros(128)
    flat[:64] = 1.0
    opt = optim.Adam(flat)
    for _ in range(3):
        g = torch.zeros(128)
        g[:64] = 0.5
        opt.update_(flat, g)
    assert torch.all(flat[64:] == 0.0) and torch.all(flat[:64] < 1.0)
