"""Evaluation of a trained wavefunction: the reference's evaluation loop and its summary
statistics, including the autocorrelation-corrected uncertainty of the energy.

``evaluate_wavefunction`` mirrors ``optimization/evaluation.py:117-201`` for the energy
observable: burn-in, then per evaluation epoch the inter-steps of Metropolis-Hastings and the
local energies of all walkers, whose FP64 mean (``dw_energy_stats``) and variance form the
history. ``summarize`` is the summary of ``evaluation.py:260-268``: per metric the nan-mean over
epochs, sigma = nan-std / sqrt(N) and, for scalar histories, sigma_corr = sigma sqrt(2 tau) with
the autocorrelation time tau of ``utils/utils.py:514-546``, restated step by step (including its
fit of 1 - log(ac) through the origin over the shifts before the first autocorrelation below the
threshold).
"""
from __future__ import annotations

import dataclasses
from typing import Dict, Iterable, Optional

import numpy as np


def autocorrelation(x: Iterable[float], n_shifts: int = 50) -> np.ndarray:
    """Normalised autocorrelation of a 1-D series for shifts 0 .. min(n_shifts, len/2) - 1
    (``utils/utils.py:514-524``): shift i correlates x[i:] with x[:-i], each centred and scaled by
    its own mean and standard deviation; shift 0 is 1."""
    x = np.asarray(x, dtype=np.float64)
    if x.ndim != 1:
        raise ValueError("autocorrelation expects a 1-D series")
    n = min(n_shifts, len(x) // 2)
    ac = np.ones(n)
    for i in range(1, n):
        a, b = x[i:], x[:-i]
        ac[i] = np.mean((a - a.mean()) * (b - b.mean())) / (a.std() * b.std())
    return ac


def autocorrelation_time(x: Iterable[float], n_shifts: int = 50, ac_threshold: float = 0.01) -> float:
    """Decay time of the autocorrelation (``utils/utils.py:527-546``): the shifts before the first
    autocorrelation below `ac_threshold` are fitted as y = 1 - log(ac) = t / tau through the
    origin, tau = sum t^2 / sum t y; a single usable shift gives 0.5."""
    ac = autocorrelation(x, n_shifts)
    noise = ac < ac_threshold
    n_fit = int(np.argmax(noise)) if np.any(noise) else len(ac)
    if n_fit == 1:
        return 0.5
    t = np.arange(n_fit, dtype=np.float64)
    y = 1.0 - np.log(ac[:n_fit])
    return float(np.sum(t ** 2) / np.sum(t * y))


def summarize(history: Dict[str, Iterable]) -> Dict[str, float]:
    """Per metric: mean, ``_sigma`` and (1-D histories) ``_sigma_corr`` (evaluation.py:260-268)."""
    out: Dict[str, float] = {}
    for key, h in history.items():
        h = np.asarray(h, dtype=np.float64)
        out[key] = np.nanmean(h, axis=0)
        out[key + "_sigma"] = np.nanstd(h, axis=0) / np.sqrt(len(h))
        if h.ndim == 1:
            out[key + "_sigma_corr"] = out[key + "_sigma"] * np.sqrt(2.0 * autocorrelation_time(h))
    return out


@dataclasses.dataclass
class ForceEvaluationConfig:
    """ForceEvaluationConfig (configuration.py:1225-1229)."""

    use: bool = True
    R_cut: float = 0.1
    R_core: float = 0.5
    use_antithetic_sampling: bool = False


def force_metrics(forces: np.ndarray) -> Dict[str, np.ndarray]:
    """The force observables of get_observables (evaluation.py:152-157): calculate_forces returns
    the [n_ions, 3] batch mean, and the metrics are its nanmean and nan-variance over axis 0."""
    f = np.asarray(forces, dtype=np.float64)
    mean = np.nanmean(f, axis=0)
    return {"forces_mean": mean, "forces_var": np.nanmean((f - mean) ** 2, axis=0)}


def evaluate_wavefunction(params, state, mcmc, n_epochs: int, n_burn_in: Optional[int] = None,
                          n_inter_steps: Optional[int] = None, group=None,
                          forces: Optional[ForceEvaluationConfig] = None):
    """Burn-in, then `n_epochs` x (inter-steps, local energies); returns (history, summary, state).

    history: per epoch ``E_mean`` (FP64 mean of the walkers' local energies) and ``E_var``; with
    several ranks both are combined as the reference's pmean (evaluation.py:148-151). With a
    force configuration also ``forces_mean`` / ``forces_var`` (evaluation.py:152-157) from
    dw_forces at the chain's current log psi^2, averaged over ranks."""
    from . import api, dist
    a = params.arch
    spin = (a.n_up, a.n_dn)
    burn = mcmc.config.n_burn_in if n_burn_in is None else n_burn_in
    inter = mcmc.config.n_inter_steps if n_inter_steps is None else n_inter_steps
    if burn > 0:
        mcmc.run_mcmc_steps(None, state, params, a.n_up, a.n_dn, None, n_steps=burn, reevaluate=True, group=group)
    hist: Dict[str, list] = {"E_mean": [], "E_var": []}
    if forces is not None and forces.use:
        hist["forces_mean"], hist["forces_var"] = [], []
    for _ in range(n_epochs):
        mcmc.run_mcmc_steps(None, state, params, a.n_up, a.n_dn, None, n_steps=inter, reevaluate=True, group=group)
        E = api.local_energy(params, spin, state.r, state.R, state.Z)
        st = api.energy_stats(E)
        m, v = dist.combine_moments(st[0], st[1], group)
        hist["E_mean"].append(float(m))
        hist["E_var"].append(float(v))
        if "forces_mean" in hist:
            F = api.calculate_forces(params, state.r, state.R, state.Z, state.log_psi_sqr, forces.R_cut, forces.R_core,
                                     forces.use_antithetic_sampling)
            fm = force_metrics(F.cpu().numpy())
            hist["forces_mean"].append(dist.pmean_array(fm["forces_mean"], group))
            hist["forces_var"].append(dist.pmean_array(fm["forces_var"], group))
    return hist, summarize(hist), state
