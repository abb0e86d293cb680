"""Walker-sharded execution over several ranks: the cross-rank reductions of the VMC loop.

The reference shards the walkers over devices with ``jax.pmap`` and combines them with
``pmean`` (``utils/utils.py:28-30``) at four places:

* the Metropolis-Hastings acceptance rate, every step (``mcmc.py:367``);
* the energy mean and variance (``optimization/loss_function.py:94-99``);
* the clipping centre and width (``loss_function.py:19-30``);
* the gradients (``optimizers.py:133``).

Here every rank (one process per GPU, ``torch.distributed``) runs the single-GPU kernels on its
own walkers, and the functions below combine the per-rank results with all-reduces (NCCL
between GPUs, gloo in the CPU tests). ``pmean`` is the plain mean of the per-rank values, as in
the reference: ranks are not weighted by their walker counts, and a rank whose energies are all
NaN makes the mean NaN. With one rank (or without an initialised process group) every function
is the identity.
"""
from __future__ import annotations

from typing import Tuple

import torch

# DwMcmcScalars starts with the two FP64 fields acc_rate and last_acc (include/dwgb.h).
_SCALAR_FP64_FIELDS = 2


def world(group=None) -> int:
    """Number of ranks of `group` (1 when torch.distributed is not initialised)."""
    if not (torch.distributed.is_available() and torch.distributed.is_initialized()):
        return 1
    return torch.distributed.get_world_size(group)


def pmean_(t: torch.Tensor, group=None) -> torch.Tensor:
    """In-place mean over ranks (all-reduce sum, then divide)."""
    w = world(group)
    if w > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.SUM, group=group)
        t.div_(w)
    return t


def pmean_array(x, group=None, device=None):
    """pmean of a small host array (e.g. the force metrics), returned as float64 numpy; the
    exchange runs on `device` (the backend's device: CUDA under NCCL, CPU under gloo)."""
    import numpy as np
    a = np.asarray(x, dtype=np.float64)
    if world(group) == 1:
        return a
    if device is None:
        device = "cuda" if torch.distributed.get_backend(group) == "nccl" else "cpu"
    t = torch.as_tensor(a, device=device).clone()
    pmean_(t, group)
    return t.cpu().numpy()


def combine_moments(mean: torch.Tensor, var: torch.Tensor, group=None) -> Tuple[torch.Tensor, torch.Tensor]:
    """Global (pmean of means, pmean of nanmean((x - global mean)^2)) from each rank's nanmean and
    population variance, as ``E_mean = pmean(nanmean(E))``,
    ``E_var = pmean(nanmean((E - E_mean)^2))`` (loss_function.py:94-95, :20-28). On one rank the
    nanmean of (x - m)^2 is var + (mean - m)^2. Returns FP64 scalars on the input's device."""
    m = mean.detach().to(torch.float64).reshape(1).clone()
    pmean_(m, group)
    v = (var.detach().to(torch.float64).reshape(1) + (mean.detach().to(torch.float64).reshape(1) - m) ** 2).clone()
    pmean_(v, group)
    return m[0], v[0]


def sync_chain_scalars_(scalars: torch.Tensor, group=None) -> torch.Tensor:
    """Averages the running acceptance rate and the last step's acceptance of a DwMcmcScalars
    device struct (a uint8 tensor) over ranks, in place. Called after every MH step: the kernel
    has just applied acc_rate <- 0.9 acc_rate + 0.1 mean(accepted) with its own walkers, and the
    mean over ranks of that update is 0.9 acc_rate + 0.1 pmean(mean(accepted)) (mcmc.py:367-371)
    because acc_rate was equal on all ranks before the step. The step-size rule reads the
    acc_rate before the update, so all ranks also keep equal step sizes."""
    if world(group) > 1:
        f = scalars[: 8 * _SCALAR_FP64_FIELDS].view(torch.float64)
        pmean_(f, group)
    return scalars


def sharded_clipped_gradient(E: torch.Tensor, clipping_state, clip_by: float, from_previous_step: bool,
                             stats_fn, clip_fn, backward_fn, group=None):
    """The clipped VMC gradient over walkers sharded across ranks (loss_function.py:60-156).

    stats_fn(E) -> (nanmean, population variance) of this rank's energies;
    clip_fn(E, center, width) -> (E_clip, nanmean, population variance of E_clip);
    backward_fn(coeff) -> sum_b coeff_b d log psi^2_b / d theta for this rank's walkers.
    Per rank the gradient is (1/B_rank) sum_b d log psi^2_b (E_clip,b - E_mean_clipped) with the
    global clipped mean, then pmean over ranks; the next clipping state comes from the clipped
    energies (loss_function.py:70-71). Returns (loss, new_state, aux, grads)."""
    e_mean_loc, e_var_loc = stats_fn(E)
    E_mean, E_var = combine_moments(e_mean_loc, e_var_loc, group)
    center, width = clipping_state
    if not from_previous_step:
        center, width = float(E_mean), float(E_var) ** 0.5 * clip_by
    E_clip, c_mean_loc, c_var_loc = clip_fn(E, center, width)
    Ec_mean, Ec_var = combine_moments(c_mean_loc, c_var_loc, group)
    B = E.numel()
    coeff = (E_clip.to(torch.float64) - Ec_mean) / B
    grads = backward_fn(coeff)
    pmean_(grads, group)
    new_state = (float(Ec_mean), float(Ec_var) ** 0.5 * clip_by)
    aux = dict(E_mean=E_mean, E_var=E_var, E_mean_clipped=Ec_mean, E_var_clipped=Ec_var, E_loc_clipped=E_clip,
               E_loc=E)
    return Ec_mean, new_state, aux, grads
