"""Evaluation statistics and loop (no GPU): autocorrelation and its decay time as
utils/utils.py:514-546 computes them (known-answer cases, an AR(1) chain), the summary of
optimization/evaluation.py:260-268, and the loop order of evaluation.py:117-201 over stand-ins."""
import types

import numpy as np
import pytest
import torch

from deeperwin_gb300 import evaluation as EV


def test_autocorrelation_known_answers():
    x = np.arange(1.0, 7.0)                                  # linear: every shift correlates perfectly
    np.testing.assert_allclose(EV.autocorrelation(x), [1.0, 1.0, 1.0])
    assert EV.autocorrelation_time(x) == pytest.approx(5.0 / 3.0)       # sum t^2 / sum t, t = 0, 1, 2
    alt = np.tile([1.0, -1.0], 5)                            # first shift anti-correlated: below threshold
    assert EV.autocorrelation(alt)[1] == pytest.approx(-1.0)
    assert EV.autocorrelation_time(alt) == 0.5
    assert len(EV.autocorrelation(np.random.default_rng(0).standard_normal(300))) == 50


def test_autocorrelation_time_of_ar1_chain():
    rho, n = 0.9, 400_000
    rng = np.random.default_rng(1)
    e = rng.standard_normal(n)
    x = np.empty(n)
    x[0] = e[0]
    for i in range(1, n):
        x[i] = rho * x[i - 1] + np.sqrt(1 - rho ** 2) * e[i]
    ac = EV.autocorrelation(x)
    np.testing.assert_allclose(ac[:10], rho ** np.arange(10), atol=0.01)
    # the reference's fit on the exact autocorrelation rho^t: shifts until rho^t < 0.01, y = 1 - log ac
    n_fit = int(np.argmax(rho ** np.arange(50) < 0.01))
    t = np.arange(n_fit)
    tau_exact_ac = np.sum(t ** 2) / np.sum(t * (1 - t * np.log(rho)))
    assert EV.autocorrelation_time(x) == pytest.approx(tau_exact_ac, rel=0.1)


def test_summary():
    rng = np.random.default_rng(2)
    h = {"E_mean": rng.normal(-1.0, 0.1, 200), "forces": rng.normal(0.0, 1.0, (200, 3))}
    h["E_mean"][5] = np.nan
    s = EV.summarize(h)
    m = h["E_mean"]
    assert s["E_mean"] == pytest.approx(np.nanmean(m))
    assert s["E_mean_sigma"] == pytest.approx(np.nanstd(m) / np.sqrt(200))
    assert "forces_sigma_corr" not in s and s["forces_sigma"].shape == (3,)
    clean = np.where(np.isnan(m), 0.0, m)
    assert np.isfinite(s["E_mean_sigma"])
    s2 = EV.summarize({"E": clean})
    assert s2["E_sigma_corr"] == pytest.approx(s2["E_sigma"] * np.sqrt(2 * EV.autocorrelation_time(clean)))


def test_evaluation_loop_order(monkeypatch):
    from deeperwin_gb300 import api
    calls = []
    energies = iter([torch.tensor([1.0, 2.0, 3.0]), torch.tensor([2.0, 2.0, 2.0]), torch.tensor([0.0, 4.0, 5.0])])

    class MH:
        config = types.SimpleNamespace(n_burn_in=7, n_inter_steps=3)

        def run_mcmc_steps(self, func, state, params, n_up, n_dn, fixed, n_steps, reevaluate, group=None):
            calls.append(("mcmc", n_steps, reevaluate))
            return state

    def fake_le(params, spin, r, R, Z):
        calls.append(("E",))
        return next(energies)

    def fake_stats(E):
        x = E.double()
        return torch.stack([x.mean(), x.var(unbiased=False), torch.tensor(float(len(x)), dtype=torch.float64)])

    monkeypatch.setattr(api, "local_energy", fake_le)
    monkeypatch.setattr(api, "energy_stats", fake_stats)
    params = types.SimpleNamespace(arch=types.SimpleNamespace(n_up=1, n_dn=1))
    state = types.SimpleNamespace(r=None, R=None, Z=None)
    hist, summ, _ = EV.evaluate_wavefunction(params, state, MH(), n_epochs=3)
    assert calls == [("mcmc", 7, True), ("mcmc", 3, True), ("E",), ("mcmc", 3, True), ("E",), ("mcmc", 3, True), ("E",)]
    np.testing.assert_allclose(hist["E_mean"], [2.0, 2.0, 3.0])
    np.testing.assert_allclose(hist["E_var"], [2.0 / 3.0, 0.0, 14.0 / 3.0])
    assert summ["E_mean"] == pytest.approx(7.0 / 3.0)


def test_force_metrics_and_loop(monkeypatch):
    """Force observables as get_observables forms them (evaluation.py:152-157): nanmean and
    nan-variance over axis 0 of calculate_forces' [n_ions, 3] result, once per epoch after the
    energies."""
    from deeperwin_gb300 import api
    F = np.array([[1.0, 2.0, 3.0], [3.0, np.nan, -1.0]])
    m = EV.force_metrics(F)
    np.testing.assert_allclose(m["forces_mean"], [2.0, 2.0, 1.0])
    np.testing.assert_allclose(m["forces_var"], [1.0, 0.0, 4.0])
    calls = []

    class MH:
        config = types.SimpleNamespace(n_burn_in=0, n_inter_steps=2)

        def run_mcmc_steps(self, func, state, params, n_up, n_dn, fixed, n_steps, reevaluate, group=None):
            calls.append("mcmc")
            return state

    monkeypatch.setattr(api, "local_energy", lambda *a, **k: (calls.append("E"), torch.tensor([1.0, 3.0]))[1])
    monkeypatch.setattr(api, "energy_stats", lambda E: torch.tensor([2.0, 1.0, 2.0], dtype=torch.float64))

    def fake_forces(params, r, R, Z, lp, R_cut, R_core, anti):
        calls.append(("F", R_cut, R_core, anti))
        return torch.as_tensor(F)
    monkeypatch.setattr(api, "calculate_forces", fake_forces)
    params = types.SimpleNamespace(arch=types.SimpleNamespace(n_up=1, n_dn=1))
    state = types.SimpleNamespace(r=None, R=None, Z=None, log_psi_sqr=None)
    cfg = EV.ForceEvaluationConfig(R_cut=0.2, use_antithetic_sampling=True)
    hist, summ, _ = EV.evaluate_wavefunction(params, state, MH(), n_epochs=2, forces=cfg)
    assert calls == ["mcmc", "E", ("F", 0.2, 0.5, True), "mcmc", "E", ("F", 0.2, 0.5, True)]
    np.testing.assert_allclose(summ["forces_mean"], [2.0, 2.0, 1.0])
    assert summ["forces_mean_sigma"].shape == (3,)
