"""VMC gradient: the hand-written d log psi^2 / d theta backward behind torch.autograd.

Mirrors ``build_value_and_grad_func`` (optimization/loss_function.py:75-156): the loss is the
(tanh-clipped) mean local energy and its gradient is
    (1/B) sum_b d/dtheta log psi^2_b * (E_clip,b - mean E_clip) = 2 E[(E - <E>) grad log|psi|],
formed on the GPU by dw_log_psi_sqr_backward, which recomputes the forward activations.
"""
from __future__ import annotations

import ctypes
import dataclasses
from typing import Tuple

import torch

from . import _lib
from . import dist
from .api import Params, _WS, _geometry, _ptr, _stream, local_energy


def log_psi_sqr_backward(params: Params, r: torch.Tensor, R, Z, coeff: torch.Tensor) -> torch.Tensor:
    """d/dtheta sum_b coeff_b log psi^2_b as a packed float32 vector (the params layout)."""
    a = params.arch
    dev = params.flat.device
    r = r.to(device=dev, dtype=torch.float32).contiguous()
    coeff = coeff.to(device=dev, dtype=torch.float32).contiguous()
    B = r.shape[0]
    Rt, Zt = (R, Z) if torch.is_tensor(R) and R.is_cuda else _geometry(R, Z, dev)
    grad = torch.zeros_like(params.flat)
    L = _lib.lib()
    nbytes = L.dw_workspace_bytes(ctypes.byref(params.c_arch), params.prec, B, 3)
    ws = _WS.get("bwd", nbytes, dev)
    _lib.check(L.dw_log_psi_sqr_backward(ctypes.byref(params.c_arch), params.prec, _ptr(params.flat),
                                         _ptr(params.prepared), _ptr(r), B, _ptr(Rt), _ptr(Zt), _ptr(coeff),
                                         _ptr(grad), _ptr(ws), nbytes, _stream()), "dw_log_psi_sqr_backward")
    return grad


class LogPsiSqr(torch.autograd.Function):
    """log psi^2(theta; r) with theta the packed parameter vector; backward by the CUDA kernel."""

    @staticmethod
    def forward(ctx, flat: torch.Tensor, params: Params, r: torch.Tensor, R, Z):
        from .api import log_psi_sqr
        ctx.params, ctx.R, ctx.Z = params, R, Z
        ctx.save_for_backward(r)
        a = params.arch
        _, lp = log_psi_sqr(params, a.n_up, a.n_dn, r, R, Z)
        return lp

    @staticmethod
    def backward(ctx, g: torch.Tensor):
        (r,) = ctx.saved_tensors
        grad = log_psi_sqr_backward(ctx.params, r, ctx.R, ctx.Z, g)
        return grad, None, None, None, None


def log_psi_sqr_autograd(params: Params, r, R, Z) -> torch.Tensor:
    return LogPsiSqr.apply(params.flat, params, r, R, Z)


@dataclasses.dataclass
class ClippingConfig:
    """ClippingConfig defaults (configuration.py:1052-1058): tanh, std width, mean center, x5."""

    name: str = "tanh"
    width_metric: str = "std"
    center: str = "mean"
    from_previous_step: bool = True
    clip_by: float = 5.0


def init_clipping_state() -> Tuple[float, float]:
    """(center, width) = (0, 1e12) (loss_function.py:12-16)."""
    return (0.0, 1e12)


def _clip(E: torch.Tensor, center: float, width: float, clip_by: float):
    out = torch.empty(4, dtype=torch.float64, device=E.device)
    Ec = torch.empty_like(E)
    _lib.check(_lib.lib().dw_clip_energies(_ptr(E.contiguous()), E.numel(), float(center), float(width),
                                           float(clip_by), _ptr(Ec), _ptr(out), _stream()), "dw_clip_energies")
    return Ec, out


def build_value_and_grad_func(log_psi_sqr_func=None, get_local_energy=None, clipping_config: ClippingConfig = None,
                              is_complex: bool = False, kfac_register_complex: bool = False, group=None):
    """Returns value_and_grad(params, clipping_state, spin_state, batch) ->
    ((loss, (clipping_state, aux)), grads) like the reference's jax.value_and_grad(total_energy).

    With several ranks (torch.distributed initialised; `group` or the default group) each rank
    passes its own walkers and the energy statistics, clipping state and gradients are combined
    across ranks as the reference's pmean does (see deeperwin_gb300.dist)."""
    if is_complex:
        raise NotImplementedError("only real-valued wavefunctions are supported")
    cfg = clipping_config or ClippingConfig()
    if cfg.name != "tanh" or cfg.width_metric != "std" or cfg.center != "mean":
        raise NotImplementedError("tanh clipping with mean center and std width is implemented")

    def value_and_grad(params: Params, clipping_state, spin_state, batch):
        r, R, Z = batch[:3]
        E = local_energy(params, spin_state, r, R, Z)
        from .api import energy_stats
        if dist.world(group) > 1:
            def stats_fn(e):
                s = energy_stats(e)
                return s[0], s[1]

            def clip_fn(e, c, w):
                ec, o = _clip(e, c, w, cfg.clip_by)
                return ec, o[0], o[1]

            loss, new_state, aux, grads = dist.sharded_clipped_gradient(
                E, clipping_state, cfg.clip_by, cfg.from_previous_step, stats_fn, clip_fn,
                lambda coeff: log_psi_sqr_backward(params, r, R, Z, coeff.float()), group)
            return (loss, (new_state, aux)), grads
        st = energy_stats(E)
        center, width = clipping_state
        if not cfg.from_previous_step:
            center, width = float(st[0]), float(st[1]) ** 0.5 * cfg.clip_by
        E_clip, cs = _clip(E, center, width, cfg.clip_by)
        B = E.numel()
        coeff = (E_clip.double() - cs[0]) / B
        grads = log_psi_sqr_backward(params, r, R, Z, coeff.float())
        aux = dict(E_mean=st[0], E_var=st[1], E_mean_clipped=cs[0], E_var_clipped=cs[1], E_loc_clipped=E_clip,
                   E_loc=E)
        new_state = (float(cs[2]), float(cs[3]))
        return (cs[0], (new_state, aux)), grads

    return value_and_grad
